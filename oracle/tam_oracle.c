/*
 * tam_oracle.c -- CPU FP64 oracle (TEST INFRASTRUCTURE ONLY).
 *
 * Restates the reference Fortran hot paths in C, each function citing the
 * file:line it follows.  Compile with -ffp-contract=off so no multiply-add
 * is fused (the reference's arithmetic is evaluated statement by statement).
 * See tam_oracle.h for the parity status of this oracle.
 */
#include "tam_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* src/constants.f90:13 -- truncated constants, promoted to FP64 by -freal-4-real-8 */
#define PI_R    3.141592
#define TWOPI_R 6.283185

/* src/thermalConst_mod.f90:5-6 */
#define AIR_HEAT_CAP 1.006e3
#define LW 2256.e3
#define WATER_INIT 0.75
#define PROTEIN (1.0 - WATER_INIT)

/* --------------------------------------------------------------- Philox -- */
#define PHILOX_M0 0xD2511F53u
#define PHILOX_M1 0xCD9E8D57u
#define PHILOX_W0 0x9E3779B9u
#define PHILOX_W1 0xBB67AE85u

/* Philox4x32-10, Salmon, Moraes, Dror & Shaw, "Parallel random numbers: as
 * easy as 1, 2, 3", SC'11: ten rounds of two 32x32->64 multiplies with the
 * Weyl key schedule. */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4])
{
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)PHILOX_M0 * c0;
        uint64_t p1 = (uint64_t)PHILOX_M1 * c2;
        uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
        uint32_t n1 = (uint32_t)p1;
        uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
        uint32_t n3 = (uint32_t)p0;
        c0 = n0; c1 = n1; c2 = n2; c3 = n3;
        k0 += PHILOX_W0; k1 += PHILOX_W1;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

void orc_philox_uniform4(uint64_t seed, uint64_t pid, uint32_t stream, uint32_t ev, double u[4])
{
    uint32_t ctr[4] = {ev, (uint32_t)pid, (uint32_t)(pid >> 32), stream};
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    uint32_t x[4];
    orc_philox4x32_10(ctr, key, x);
    for (int i = 0; i < 4; ++i) u[i] = ((double)x[i] + 0.5) * 0x1p-32;
}

/* ------------------------------------------------- thermal constants -- */
/* src/thermalConst_mod.f90:11-25 (the T<0 `error stop` is reported by callers) */
double orc_air_thermal_cond(double T)
{
    const double a = -0.188521, b = 0.000367259, c = 0.212453;
    return a * exp(-(b * (T - 273.15))) + c;
}
/* src/thermalConst_mod.f90:28-38 */
double orc_air_density(double T) { return 101.325e3 / (287.058 * T); }
/* src/thermalConst_mod.f90:41-50 */
double orc_water_content(double Q, double w, double QVapor)
{
    double a = WATER_INIT - WATER_INIT * (Q / QVapor);
    double m = a < WATER_INIT ? a : WATER_INIT;
    m = m < w ? m : w;
    return m > 0.0 ? m : 0.0;
}
/* src/thermalConst_mod.f90:54-62 */
double orc_skin_density(double w) { return 1000.0 / (w + 0.649 * PROTEIN); }
/* src/thermalConst_mod.f90:65-73 */
double orc_skin_heat_cap(double w) { return 1000.0 * (4.2 * w + 1.09 * PROTEIN); }
/* src/thermalConst_mod.f90:76-84 */
double orc_skin_thermal_cond(double w, double rho) { return rho * (6.28e-4 * w + 1.17e-4 * PROTEIN); }

/* ------------------------------------------------------ layout helpers -- */
#define HX(s) ((int64_t)(s)->p.nx + 2)
#define HY(s) ((int64_t)(s)->p.ny + 2)
#define HZ(s) ((int64_t)(s)->p.nz + 2)
#define IH(s, i, j, k) ((int64_t)(i) + HX(s) * ((int64_t)(j) + HY(s) * (int64_t)(k)))
#define II(s, i, j, k) ((int64_t)((i)-1) + (int64_t)(s)->p.nx * ((int64_t)((j)-1) + (int64_t)(s)->p.ny * (int64_t)((k)-1)))

static int64_t n_halo(const orc_ref_state *s) { return HX(s) * HY(s) * HZ(s); }
static int64_t n_int(const orc_ref_state *s) { return (int64_t)s->p.nx * s->p.ny * s->p.nz; }

static double *dalloc(int64_t n)
{
    double *p = (double *)calloc((size_t)(n > 0 ? n : 1), sizeof(double));
    return p;
}

static int nthr(int n)
{
#ifdef _OPENMP
    return n > 0 ? n : omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}

/* ------------------------------------------------------ getPwr family -- */
/* src/3dFD.f90:365-377 */
static double pwr_gaussian(const orc_ref_state *s)
{
    double fact = 2. * sqrt(2. * log(2.));
    double mu = fact * s->pulseLength;
    double sig = s->pulseLength / fact;
    double tm = s->time - mu;
    return s->p.power * exp(-((tm * tm) / (2.0 * (sig * sig))));
}
/* src/3dFD.f90:380-392 */
static double pwr_tophat(const orc_ref_state *s) { return s->laser_flag ? s->p.power : 0.0; }
/* src/3dFD.f90:395-421 */
static double pwr_triangular(orc_ref_state *s)
{
    double m = s->p.power / s->pulseLength;
    double c = 2.0 * s->p.power;
    double P;
    if (!s->laser_flag) return 0.0;
    if (s->pulseFlag) {
        P = -m * s->time + c;
        if (P < 0.0) P = 0.0;
    } else if (s->time >= s->pulseLength) {
        s->pulseFlag = 1;
        P = -m * s->time + c;
        if (P < 0.0) P = 0.0;
    } else {
        P = m * s->time;
    }
    return P;
}
double orc_ref_get_pwr(orc_ref_state *s)
{
    switch (s->p.pulse_type) {
    case ORC_PULSE_GAUSSIAN: return pwr_gaussian(s);
    case ORC_PULSE_TOPHAT: return pwr_tophat(s);
    default: return pwr_triangular(s);
    }
}

/* ----------------------------------------------- initThermalCoeff etc. -- */
/* src/3dFD.f90:233-309 (numpoints generalised to nx, ny, nz per axis) */
static int init_thermal(orc_ref_state *s)
{
    const orc_ref_params *p = &s->p;
    s->dx = (2.0 * p->xmax * 1.e-2) / (p->nx + 2.0);
    s->dy = (2.0 * p->ymax * 1.e-2) / (p->ny + 2.0);
    s->dz = (2.0 * p->zmax * 1.e-2) / (p->nz + 2.0);

    int64_t nh = n_halo(s), ni = n_int(s);
    for (int64_t q = 0; q < ni; ++q) { s->Q[q] = 0.0; s->water[q] = WATER_INIT; }
    s->skinDensityInit = orc_skin_density(WATER_INIT);
    double heatCaptmp = orc_skin_heat_cap(WATER_INIT);
    double densitytmp = orc_skin_density(WATER_INIT);
    double kappatmp = orc_skin_thermal_cond(WATER_INIT, densitytmp);
    double alphatmp = kappatmp / (densitytmp * orc_skin_heat_cap(WATER_INIT));

    double alpha_air = orc_air_thermal_cond(25.0 + 273.0) / (orc_air_density(25.0 + 273.0) * AIR_HEAT_CAP);
    double kair = orc_air_thermal_cond(25. + 273.);
    double ktis = orc_skin_thermal_cond(WATER_INIT, densitytmp);
    for (int64_t q = 0; q < nh; ++q) {
        s->alpha[q] = alphatmp;
        s->kappa[q] = kair;
        s->density[q] = densitytmp;
        s->heatcap[q] = heatCaptmp;
        s->coeff[q] = 0.0;
    }
    /* alpha(:,:,nzg+1) = air (3dFD.f90:272) */
    for (int j = 0; j <= p->ny + 1; ++j)
        for (int i = 0; i <= p->nx + 1; ++i) s->alpha[IH(s, i, j, p->nz + 1)] = alpha_air;
    double constd = (1.0 / (s->dx * s->dx)) + (1.0 / (s->dy * s->dy)) + (1.0 / (s->dz * s->dz));
    s->delt = 1.0 / (1.0 * alphatmp * constd);
    double cint = alphatmp * s->delt / kappatmp;
    for (int k = 1; k <= p->nz; ++k)
        for (int j = 1; j <= p->ny; ++j)
            for (int i = 1; i <= p->nx; ++i) {
                s->kappa[IH(s, i, j, k)] = ktis;
                s->coeff[IH(s, i, j, k)] = cint;
            }
    s->pulseLength = (p->energy_per_pixel * 1.e-3 * (double)(9 * 9)) / p->power;
    s->volumeVoxel = (2.0 * p->xmax * 1.e-2 / p->nx) * (2.0 * p->ymax * 1.e-2 / p->ny) * (2.0 * p->zmax * 1.e-2 / p->nz);
    s->massVoxel = densitytmp * s->volumeVoxel;
    s->QVapor = LW * s->massVoxel;
    switch (p->pulse_type) {
    case ORC_PULSE_TOPHAT: s->realPulseLength = s->pulseLength; break;
    case ORC_PULSE_GAUSSIAN: s->realPulseLength = 20000.0 * s->pulseLength; break;
    case ORC_PULSE_TRIANGULAR: s->realPulseLength = 2.0 * s->pulseLength; break;
    default: return -1; /* error stop "no pulse type" (3dFD.f90:304-306) */
    }
    return 0;
}

orc_ref_state *orc_ref_create(const orc_ref_params *p)
{
    orc_ref_state *s = (orc_ref_state *)calloc(1, sizeof(orc_ref_state));
    if (!s) return NULL;
    s->p = *p;
    if (s->p.numproc < 1) s->p.numproc = 1;
    int64_t nh = n_halo(s), ni = n_int(s);
    /* alloc_array + zarray (src/subs.f90:27-77) */
    s->xface = dalloc(p->nx + 2);
    s->yface = dalloc(p->ny + 2);
    s->zface = dalloc(p->nz + 2);
    s->rhokap = dalloc(nh);
    s->jmean = dalloc(ni);
    s->jmeanGLOBAL = dalloc(ni);
    s->tissue = dalloc(ni);
    s->temp = dalloc(nh);
    s->thres = dalloc(3 * ni);
    s->kappa = dalloc(nh);
    s->density = dalloc(nh);
    s->heatcap = dalloc(nh);
    s->coeff = dalloc(nh);
    s->alpha = dalloc(nh);
    s->Q = dalloc(ni);
    s->water = dalloc(ni);
    if (!s->xface || !s->yface || !s->zface || !s->rhokap || !s->jmean || !s->jmeanGLOBAL || !s->tissue ||
        !s->temp || !s->thres || !s->kappa || !s->density || !s->heatcap || !s->coeff || !s->alpha || !s->Q ||
        !s->water) {
        orc_ref_free(s);
        return NULL;
    }
    /* mcpolar.f90:66-73 */
    s->time = 0.; s->pulseCount = 0.; s->repetitionCount = 0.; s->laserOn = 1.;
    s->laser_flag = 1; s->pulseFlag = 0; s->counter = 0; s->pulsesDone = 0;
    /* init_opt1 (src/ch_opt.f90:7-25) */
    s->hgg = 0.9;
    s->g2 = s->hgg * s->hgg;
    s->mu_water = 510.0;
    s->mu_protein = 170.0;
    s->mua = s->mu_water + s->mu_protein;
    s->mus = 0.;
    s->kappa_opt = s->mus + s->mua;
    s->albedo = s->mus / s->kappa_opt;
    /* gridset (src/gridset.f90:23-45): faces in a shifted frame [0, 2max] */
    for (int i = 1; i <= p->nx + 1; ++i) s->xface[i] = (i - 1) * 2. * p->xmax / p->nx;
    for (int i = 1; i <= p->ny + 1; ++i) s->yface[i] = (i - 1) * 2. * p->ymax / p->ny;
    for (int i = 1; i <= p->nz + 1; ++i) s->zface[i] = (i - 1) * 2. * p->zmax / p->nz;
    for (int k = 1; k <= p->nz; ++k)
        for (int j = 1; j <= p->ny; ++j)
            for (int i = 1; i <= p->nx; ++i) s->rhokap[IH(s, i, j, k)] = s->kappa_opt;
    /* mcpolar.f90:112 */
    s->delta = 1.e-8 * (2. * p->zmax / p->nz);
    /* temperature init (mcpolar.f90:123-129), in that assignment order */
    for (int64_t q = 0; q < nh; ++q) s->temp[q] = 5.0 + 273.0;
    for (int k = 0; k <= p->nz + 1; ++k)
        for (int j = 0; j <= p->ny + 1; ++j) {
            s->temp[IH(s, p->nx + 1, j, k)] = 5. + 273.;
            s->temp[IH(s, 0, j, k)] = 5. + 273.;
        }
    for (int k = 0; k <= p->nz + 1; ++k)
        for (int i = 0; i <= p->nx + 1; ++i) {
            s->temp[IH(s, i, 0, k)] = 5. + 273.;
            s->temp[IH(s, i, p->ny + 1, k)] = 5. + 273.;
        }
    for (int j = 0; j <= p->ny + 1; ++j)
        for (int i = 0; i <= p->nx + 1; ++i) {
            s->temp[IH(s, i, j, 0)] = 25. + 273.;
            s->temp[IH(s, i, j, p->nz + 1)] = 25. + 273.;
        }
    if (init_thermal(s) != 0) {
        orc_ref_free(s);
        return NULL;
    }
    /* total_time override (mcpolar.f90:134-140) */
    if (p->pulse_type == ORC_PULSE_GAUSSIAN) {
        s->p.total_time = 2. * s->pulseLength * (2. * sqrt(2. * log(2.)));
        s->realPulseLength = s->p.total_time;
    } else if ((int64_t)(s->p.total_time / s->delt) <= (int64_t)(s->realPulseLength / s->delt)) {
        s->p.total_time = s->delt * (s->realPulseLength / s->delt + 2000.);
    }
    return s;
}

void orc_ref_free(orc_ref_state *s)
{
    if (!s) return;
    free(s->xface); free(s->yface); free(s->zface); free(s->rhokap); free(s->jmean); free(s->jmeanGLOBAL);
    free(s->tissue); free(s->temp); free(s->thres); free(s->kappa); free(s->density); free(s->heatcap);
    free(s->coeff); free(s->alpha); free(s->Q); free(s->water);
    free(s);
}

/* ------------------------------------------------- reference transport -- */
/* find (src/inttau2.f90:208-239): bisection on a 1-based face array a[1..n] */
static int ref_find(double val, const double *a, int n)
{
    if (val == a[1]) return 1;
    if (val == a[n]) return n - 1;
    if ((val > a[n]) || (val < a[1])) return -1;
    int lo = 0, hi = n + 1;
    while (hi - lo > 1) {
        int mid = (hi + lo) / 2;
        if (val >= a[mid]) lo = mid;
        else hi = mid;
    }
    return lo;
}

typedef struct {
    double nxp, nyp, nzp;
} refdir;

/* wall_dist (src/inttau2.f90:75-121) */
static double ref_wall_dist(const orc_ref_state *s, int ci, int cj, int ck, double xc, double yc, double zc,
                            const refdir *d, int *dir)
{
    double dx, dy, dz;
    if (d->nxp > 0.) dx = (s->xface[ci + 1] - xc) / d->nxp;
    else if (d->nxp < 0.) dx = (s->xface[ci] - xc) / d->nxp;
    else dx = 100000.;
    if (d->nyp > 0.) dy = (s->yface[cj + 1] - yc) / d->nyp;
    else if (d->nyp < 0.) dy = (s->yface[cj] - yc) / d->nyp;
    else dy = 100000.;
    if (d->nzp > 0.) dz = (s->zface[ck + 1] - zc) / d->nzp;
    else if (d->nzp < 0.) dz = (s->zface[ck] - zc) / d->nzp;
    else dz = 100000.;
    double w = dx < dy ? dx : dy;
    w = w < dz ? w : dz;
    *dir = 0;
    if (w == dx) *dir = 1;
    if (w == dy) *dir = 2;
    if (w == dz) *dir = 3;
    return w;
}

/* update_pos + update_voxels (src/inttau2.f90:124-205) */
static void ref_update_pos(const orc_ref_state *s, double *xc, double *yc, double *zc, int *ci, int *cj, int *ck,
                           double dcell, int wall, int dir, const refdir *d, double delta)
{
    if (wall) {
        if (dir == 1) {
            if (d->nxp > 0.) *xc = s->xface[*ci + 1] + delta;
            else if (d->nxp < 0.) *xc = s->xface[*ci] - delta;
            *yc = *yc + d->nyp * dcell;
            *zc = *zc + d->nzp * dcell;
        } else if (dir == 2) {
            *xc = *xc + d->nxp * dcell;
            if (d->nyp > 0.) *yc = s->yface[*cj + 1] + delta;
            else if (d->nyp < 0.) *yc = s->yface[*cj] - delta;
            *zc = *zc + d->nzp * dcell;
        } else if (dir == 3) {
            *xc = *xc + d->nxp * dcell;
            *yc = *yc + d->nyp * dcell;
            if (d->nzp > 0.) *zc = s->zface[*ck + 1] + delta;
            else if (d->nzp < 0.) *zc = s->zface[*ck] - delta;
        }
        *ci = ref_find(*xc, s->xface, s->p.nx + 1);
        *cj = ref_find(*yc, s->yface, s->p.ny + 1);
        *ck = ref_find(*zc, s->zface, s->p.nz + 1);
    } else {
        *xc = *xc + d->nxp * dcell;
        *yc = *yc + d->nyp * dcell;
        *zc = *zc + d->nzp * dcell;
    }
}

/* sourcephCO2 (src/sourceph.f90:7-49) then tauint1 (src/inttau2.f90:7-72). */
static void ref_packet(const orc_ref_state *s, uint64_t pid, uint64_t seed, uint32_t stream, double *jm)
{
    const orc_ref_params *p = &s->p;
    double u[4];
    orc_philox_uniform4(seed, pid, stream, 0u, u);
    const double spotSize = 250e-4;
    double r = u[0] * ((spotSize / 2.) * (spotSize / 2.));
    double theta = u[1] * TWOPI_R;
    double xp = sqrt(r) * cos(theta);
    double yp = sqrt(r) * sin(theta);
    double zp = p->zmax - (1.e-8 * (2. * p->zmax / p->nz));
    double phi = TWOPI_R * u[2];
    double cosp = cos(phi), sinp = sin(phi);
    double sint = 0., cost = -1.;
    refdir d = {sint * cosp, sint * sinp, cost};
    int xcell = (int)(p->nx * (xp + p->xmax) / (2. * p->xmax)) + 1;
    int ycell = (int)(p->ny * (yp + p->ymax) / (2. * p->ymax)) + 1;
    int zcell = (int)(p->nz * (zp + p->zmax) / (2. * p->zmax)) + 1;

    double xcur = xp + p->xmax, ycur = yp + p->ymax, zcur = zp + p->zmax;
    int ci = xcell, cj = ycell, ck = zcell;
    double taurun = 0., dsum = 0.;
    double tau = -log(u[3]);
    for (int64_t it = 0;; ++it) {
        int dir;
        double dcell = ref_wall_dist(s, ci, cj, ck, xcur, ycur, zcur, &d, &dir);
        double rk = s->rhokap[IH(s, ci, cj, ck)];
        double taucell = dcell * rk;
        if (taurun + taucell < tau) {
            taurun = taurun + taucell;
            dsum = dsum + dcell;
            jm[II(s, ci, cj, ck)] += dcell * rk;
            ref_update_pos(s, &xcur, &ycur, &zcur, &ci, &cj, &ck, dcell, 1, dir, &d, s->delta);
        } else {
            dcell = (tau - taurun) / rk;
            dsum = dsum + dcell;
            jm[II(s, ci, cj, ck)] += dcell * rk;
            ref_update_pos(s, &xcur, &ycur, &zcur, &ci, &cj, &ck, dcell, 0, dir, &d, s->delta);
            break;
        }
        if (ci == -1 || cj == -1 || ck == -1) break; /* tflag (inttau2.f90:58-61) */
        if (it > 100000000) break;
    }
}

void orc_ref_photons(orc_ref_state *s, int64_t p0, int64_t n, uint64_t seed, uint32_t stream, int nthreads)
{
    int T = nthr(nthreads);
    int64_t ni = n_int(s);
    if (T <= 1) {
        for (int64_t q = 0; q < n; ++q) ref_packet(s, (uint64_t)(p0 + q), seed, stream, s->jmean);
        return;
    }
    /* per-thread tallies summed in a fixed order: the role of the MPI_Allreduce at mcpolar.f90:173 */
    double *buf = (double *)calloc((size_t)T * (size_t)ni, sizeof(double));
    if (!buf) {
        for (int64_t q = 0; q < n; ++q) ref_packet(s, (uint64_t)(p0 + q), seed, stream, s->jmean);
        return;
    }
#ifdef _OPENMP
#pragma omp parallel num_threads(T)
    {
        int t = omp_get_thread_num();
        double *jm = buf + (size_t)t * (size_t)ni;
#pragma omp for schedule(static)
        for (int64_t q = 0; q < n; ++q) ref_packet(s, (uint64_t)(p0 + q), seed, stream, jm);
    }
#endif
    for (int t = 0; t < T; ++t) {
        const double *jm = buf + (size_t)t * (size_t)ni;
        for (int64_t q = 0; q < ni; ++q) s->jmean[q] += jm[q];
    }
    free(buf);
}

void orc_ref_normalise(orc_ref_state *s)
{
    const orc_ref_params *p = &s->p;
    double pw = orc_ref_get_pwr(s);
    double den = (double)(p->nphotons * (int64_t)p->numproc) * (2. * p->xmax * 1.e-2 / p->nx) *
                 (2. * p->ymax * 1.e-2 / p->ny) * (2. * p->zmax * 1.e-2 / p->nz);
    double f = (pw / 81.0) / den;
    int64_t ni = n_int(s);
    for (int64_t q = 0; q < ni; ++q) s->jmeanGLOBAL[q] = s->jmean[q] * f;
}

/* -------------------------------------------------- reference heat path -- */
/* pulse state machine (src/3dFD.f90:199-214) */
static void pulse_update(orc_ref_state *s)
{
    if (s->pulseCount >= s->realPulseLength && s->laser_flag) {
        s->laser_flag = 0;
        s->laserOn = 0.;
        s->pulseCount = 0.;
        s->pulsesDone = s->pulsesDone + 1;
        s->repetitionCount = 0.;
    } else if ((s->repetitionCount >= s->p.repetition_rate_1) && (!s->laser_flag) &&
               (s->pulsesDone < s->p.pulses_to_do)) {
        s->laser_flag = 1;
        s->laserOn = 1.;
        s->pulseCount = 0.;
        s->repetitionCount = 0.;
    }
    s->pulseCount = s->pulseCount + s->delt;
    s->repetitionCount = s->repetitionCount + s->delt;
    s->time = s->time + s->delt;
}

/* heat_sim_3D for one rank owning the whole grid (src/3dFD.f90:21-230). */
int orc_ref_heat_sim(orc_ref_state *s, int nthreads)
{
    const orc_ref_params *p = &s->p;
    int64_t nh = n_halo(s);
    double *t0 = dalloc(nh), *tn = dalloc(nh);
    if (!t0 || !tn) { free(t0); free(tn); return -2; }
    memcpy(t0, s->temp, (size_t)nh * sizeof(double));
    memcpy(tn, t0, (size_t)nh * sizeof(double));
    const double *J = s->jmeanGLOBAL;
    double *Qt = s->Q; /* scattered then gathered back unchanged in layout */

    if (s->pulseLength < s->delt) s->delt = s->pulseLength / 100.; /* 3dFD.f90:102-105 */
    s->loops_left = (int32_t)(p->total_time / ((double)p->loops * s->delt)) - s->counter;

    const double idx2 = 1.0 / (s->dx * s->dx), idy2 = 1.0 / (s->dy * s->dy), idz2 = 1.0 / (s->dz * s->dz);
    int err = 0;
    int T = nthr(nthreads);
    (void)T;
    for (int pp = 1; pp <= p->loops; ++pp) {
        const double delt = s->delt, laserOn = s->laserOn, vv = s->volumeVoxel, mv = s->massVoxel,
                     QV = s->QVapor;
#ifdef _OPENMP
#pragma omp parallel for num_threads(T) schedule(static) reduction(| : err)
#endif
        for (int k = 1; k <= p->nz; ++k)
            for (int j = 1; j <= p->ny; ++j)
                for (int i = 1; i <= p->nx; ++i) {
                    const double *K = s->kappa, *D = s->density, *C = s->heatcap;
                    int64_t c = IH(s, i, j, k);
                    int64_t zp = IH(s, i, j, k + 1), zm = IH(s, i, j, k - 1);
                    int64_t yp = IH(s, i, j + 1, k), ym = IH(s, i, j - 1, k);
                    int64_t xp = IH(s, i + 1, j, k), xm = IH(s, i - 1, j, k);
                    double kP, kM, dP, dM, cP, cM, a, d, b;
                    /* z (3dFD.f90:119-132) */
                    kP = .5 * (K[c] + K[zp]); kM = .5 * (K[c] + K[zm]);
                    dP = .5 * (D[c] + D[zp]); dM = .5 * (D[c] + D[zm]);
                    cP = .5 * (C[c] + C[zp]); cM = .5 * (C[c] + C[zm]);
                    a = 0.5 * (kM / (dM * cM)) * idz2;
                    d = 0.5 * (kP / (dP * cP)) * idz2;
                    b = 0.5 * (a + d);
                    double u_zz = a * t0[zm] - 2.0 * b * t0[c] + d * t0[zp];
                    /* y (3dFD.f90:135-148) */
                    kP = 0.5 * (K[c] + K[yp]); kM = 0.5 * (K[c] + K[ym]);
                    dP = 0.5 * (D[c] + D[yp]); dM = 0.5 * (D[c] + D[ym]);
                    cP = 0.5 * (C[c] + C[yp]); cM = 0.5 * (C[c] + C[ym]);
                    a = 0.5 * (kM / (dM * cM)) * idy2;
                    d = 0.5 * (kP / (dP * cP)) * idy2;
                    b = 0.5 * (a + d);
                    double u_yy = a * t0[ym] - 2.0 * b * t0[c] + d * t0[yp];
                    /* x (3dFD.f90:151-164) */
                    kP = .5 * (K[c] + K[xp]); kM = .5 * (K[c] + K[xm]);
                    dP = .5 * (D[c] + D[xp]); dM = .5 * (D[c] + D[xm]);
                    cP = .5 * (C[c] + C[xp]); cM = .5 * (C[c] + C[xm]);
                    a = 0.5 * (kM / (dM * cM)) * idx2;
                    d = 0.5 * (kP / (dP * cP)) * idx2;
                    b = 0.5 * (a + d);
                    double u_xx = a * t0[xm] - 2.0 * b * t0[c] + d * t0[xp];
                    /* source and boiling (3dFD.f90:166-183) */
                    int64_t q = II(s, i, j, k);
                    double tempIncrease = delt * (u_xx + u_yy + u_zz);
                    double energyIncrease = laserOn * J[q] * delt * vv + C[c] * mv * tempIncrease;
                    if (tn[c] >= 100. + 273. && Qt[q] < QV) {
                        if (energyIncrease > 0.0) {
                            double qn = Qt[q] + energyIncrease;
                            Qt[q] = qn < QV ? qn : QV;
                            tn[c] = 100.0 + 273.0;
                        } else {
                            tn[c] = tn[c] + tempIncrease + laserOn * s->coeff[c] * J[q];
                        }
                    } else {
                        tn[c] = tn[c] + tempIncrease + laserOn * s->coeff[c] * J[q];
                        if (s->temp[c] < 0.0) err |= 1; /* mpi_abort (3dFD.f90:179-182) */
                    }
                }
        memcpy(t0, tn, (size_t)nh * sizeof(double)); /* t0 = tn (3dFD.f90:187) */
        pulse_update(s);
    }
    memcpy(s->temp, t0, (size_t)nh * sizeof(double)); /* allgather back (3dFD.f90:218-222) */
    free(t0);
    free(tn);
    if (err) { s->error = 1; return -1; }
    return 0;
}

/* Arrhenius (src/3dFD.f90:424-466) */
void orc_ref_arrhenius(orc_ref_state *s)
{
    const orc_ref_params *p = &s->p;
    const double A = 3.1e98, dE = 6.3e5, R = 8.314;
    const double first = .53, second = 1.0, third = 10000.0;
    int64_t ni = n_int(s);
    for (int z = 1; z <= p->nz; ++z)
        for (int y = 1; y <= p->ny; ++y)
            for (int x = 1; x <= p->nx; ++x) {
                double T = s->temp[IH(s, x, y, z)];
                int64_t q = II(s, x, y, z);
                if (T >= 43. + 273. && T < 100.0 + 273.0 && s->rhokap[IH(s, x, y, z)] >= 0.)
                    s->tissue[q] = s->tissue[q] + s->delt * A * exp(-(dE / (R * T)));
                double *t1 = &s->thres[q], *t2 = &s->thres[q + ni], *t3 = &s->thres[q + 2 * ni];
                if (*t1 == 0.0 && s->tissue[q] >= first) *t1 = s->time;
                else if (*t2 == 0.0 && s->tissue[q] >= second) *t2 = s->time;
                else if (*t3 == 0.0 && s->tissue[q] >= third) *t3 = s->time;
            }
}

/* setupThermalCoeff (src/3dFD.f90:312-361): one sequential sweep, i fastest. */
void orc_ref_setup_thermal(orc_ref_state *s)
{
    const orc_ref_params *p = &s->p;
    int64_t ni = n_int(s);
    for (int64_t q = 0; q < ni; ++q) s->water[q] = orc_water_content(s->Q[q], s->water[q], s->QVapor);
    double *rk = s->rhokap;
    for (int k = 1; k <= p->nz; ++k)
        for (int j = 1; j <= p->ny; ++j)
            for (int i = 1; i <= p->nx; ++i) {
                int64_t c = IH(s, i, j, k), q = II(s, i, j, k);
                double T = s->temp[c];
                if (T >= p->ablate_temp + 273.0) {
                    rk[c] = 0.0;
                } else if (rk[c] > 0.) {
                    double w = s->water[q];
                    s->density[c] = orc_skin_density(w);
                    rk[c] = w * s->mu_water + s->mu_protein;
                    s->heatcap[c] = orc_skin_heat_cap(w);
                    s->kappa[c] = orc_skin_thermal_cond(w, s->density[c]);
                    s->coeff[c] = s->delt / (s->density[c] * s->heatcap[c]);
                }
                double summ = rk[IH(s, i, j, k + 1)] + rk[IH(s, i, j + 1, k)] + rk[IH(s, i + 1, j, k)] +
                              rk[IH(s, i, j, k - 1)] + rk[IH(s, i, j - 1, k)] + rk[IH(s, i - 1, j, k)];
                if (summ == 0.0) rk[c] = 0.0;
                if (rk[c] <= 0.01) {
                    if (T < 0.) s->error = 2; /* error stop in airThermalCond (thermalConst_mod.f90:20-23) */
                    s->density[c] = orc_air_density(T);
                    s->heatcap[c] = 1.006e3;
                    rk[c] = 0.;
                    s->kappa[c] = orc_air_thermal_cond(T);
                    s->alpha[c] = s->kappa[c] / (s->density[c] * s->heatcap[c]);
                    s->coeff[c] = s->delt / (orc_air_density(T) * s->heatcap[c]);
                }
            }
}

int orc_ref_outer_iteration(orc_ref_state *s, uint64_t seed, int nthreads)
{
    if (s->laser_flag) {
        /* all ranks' packets on one device: nphotons per rank x numproc ranks */
        orc_ref_photons(s, 0, s->p.nphotons * (int64_t)s->p.numproc, seed, (uint32_t)s->counter, nthreads);
        orc_ref_normalise(s);
    }
    int rc = orc_ref_heat_sim(s, nthreads);
    if (rc) return rc;
    orc_ref_arrhenius(s);
    orc_ref_setup_thermal(s);
    s->counter = s->counter + 1;
    memset(s->jmean, 0, (size_t)n_int(s) * sizeof(double));
    return s->error ? -1 : 0;
}

int64_t orc_ref_run(orc_ref_state *s, uint64_t seed, int64_t max_iters, int nthreads)
{
    int64_t it = 0;
    while (s->time <= s->p.total_time) {
        if (max_iters > 0 && it >= max_iters) break;
        int rc = orc_ref_outer_iteration(s, seed, nthreads);
        if (rc) return rc;
        ++it;
    }
    return it;
}

void orc_ref_finalize(orc_ref_state *s)
{
    const orc_ref_params *p = &s->p;
    for (int q = 1; q <= p->nx; ++q)
        for (int w = 1; w <= p->ny; ++w)
            for (int e = 1; e <= p->nz; ++e)
                if (s->rhokap[IH(s, q, w, e)] <= 0.1) s->tissue[II(s, q, w, e)] = -1.0;
}

/* --------------------------------------------------------- stokes -- */
/* src/stokes.f90:6-153.  dir = {cost, sint, phi, cosp, sinp}. */
void orc_stokes(double hgg, double g2, double u0, double u1, double dir[5])
{
    double cost = dir[0], sint = dir[1], phi = dir[2], cosp = dir[3], sinp = dir[4];
    if (hgg == 0.0) {
        cost = 2. * u0 - 1.;
        sint = (1. - cost * cost);
        if (sint <= 0.) sint = 0.;
        else sint = sqrt(sint);
        phi = TWOPI_R * u1;
        sinp = sin(phi);
        cosp = cos(phi);
    } else {
        double costp = cost, sintp = sint, phip = phi;
        double t = (1. - g2) / (1. - hgg + 2. * hgg * u0);
        double bmu = ((1. + g2) - t * t) / (2. * hgg);
        double cosb2 = bmu * bmu;
        if (fabs(bmu) > 1.) {
            if (bmu > 1.) { bmu = 1.; cosb2 = 1.; }
            else { bmu = -1.; cosb2 = 1.; }
        }
        double sinbt = sqrt(1. - cosb2);
        double ri1 = TWOPI_R * u1;
        double cosi2 = 0., sini2, cosdph;
        if (ri1 > PI_R) {
            double ri3 = TWOPI_R - ri1;
            double cosi3 = cos(ri3), sini3 = sin(ri3);
            if (bmu == 1. || bmu == -1.) goto done; /* goto 100 */
            cost = costp * bmu + sintp * sinbt * cosi3;
            if (fabs(cost) < 1.) {
                sint = fabs(sqrt(1. - cost * cost));
                sini2 = sini3 * sintp / sint;
                double bott = sint * sinbt;
                cosi2 = costp / bott - cost * bmu / bott;
            } else {
                sint = 0.;
                sini2 = 0.;
                if (cost >= 1.) cosi2 = -1.;
                if (cost <= -1.) cosi2 = 1.;
            }
            cosdph = -cosi2 * cosi3 + sini2 * sini3 * bmu;
            if (fabs(cosdph) > 1.) cosdph = cosdph > 1. ? 1. : -1.;
            phi = phip + acos(cosdph);
            if (phi > TWOPI_R) phi = phi - TWOPI_R;
            if (phi < 0.) phi = phi + TWOPI_R;
        } else {
            double cosi1 = cos(ri1), sini1 = sin(ri1);
            if (bmu == 1. || bmu == -1.) goto done;
            cost = costp * bmu + sintp * sinbt * cosi1;
            if (fabs(cost) < 1.) {
                sint = fabs(sqrt(1. - cost * cost));
                sini2 = sini1 * sintp / sint;
                double bott = sint * sinbt;
                cosi2 = costp / bott - cost * bmu / bott;
            } else {
                sint = 0.;
                sini2 = 0.;
                if (cost >= 1.) cosi2 = -1.;
                if (cost <= -1.) cosi2 = 1.;
            }
            cosdph = -cosi1 * cosi2 + sini1 * sini2 * bmu;
            if (fabs(cosdph) > 1.) cosdph = cosdph > 1. ? 1. : -1.;
            phi = phip - acos(cosdph);
            if (phi > TWOPI_R) phi = phi - TWOPI_R;
            if (phi < 0.) phi = phi + TWOPI_R;
        }
        cosp = cos(phi);
        sinp = sin(phi);
    }
    dir[0] = cost; dir[1] = sint; dir[2] = phi; dir[3] = cosp; dir[4] = sinp;
    return;
done:
    return; /* direction unchanged (stokes.f90:152) */
}

/* ------------------------------------------------------ Fresnel -- */
double orc_fresnel(double n1, double n2, double cosi)
{
    if (n1 == n2) return 0.0;
    if (cosi > 1.0) cosi = 1.0;
    double sini = sqrt(1.0 - cosi * cosi);
    double sint = n1 / n2 * sini;
    if (sint >= 1.0) return 1.0;
    double cost = sqrt(1.0 - sint * sint);
    double rs = (n1 * cosi - n2 * cost) / (n1 * cosi + n2 * cost);
    double rp = (n1 * cost - n2 * cosi) / (n1 * cost + n2 * cosi);
    return 0.5 * (rs * rs + rp * rp);
}

/* ----------------------------------------------- generic transport -- */
typedef struct {
    double mut, mua, albedo, g, g2, n;
} medprops;

static void med_lookup(const orc_mc_desc *d, const void *grid, int ix, int iy, int iz, medprops *m)
{
    if (d->medium == ORC_MED_RHOKAP) {
        const double *rk = (const double *)grid;
        int64_t hx = d->nx + 2, hy = d->ny + 2;
        double v = rk[(ix + 1) + hx * ((iy + 1) + hy * (int64_t)(iz + 1))];
        m->mut = v; m->mua = v; m->albedo = 0.0; m->g = 0.0; m->g2 = 0.0; m->n = d->rhokap_n;
    } else {
        const uint8_t *id = (const uint8_t *)grid;
        int mi = id[ix + (int64_t)d->nx * (iy + (int64_t)d->ny * iz)];
        if (mi >= d->nmat) mi = 0;
        const orc_optmat *om = &d->mat[mi];
        m->mut = om->mua + om->mus;
        m->mua = om->mua;
        m->albedo = m->mut > 0.0 ? om->mus / m->mut : 0.0;
        m->g = om->g;
        m->g2 = om->g * om->g;
        m->n = om->n;
    }
}

/* One packet of the config-mode algorithm.  Position is held as a cell index
 * plus an offset inside the cell; the event counter selects the Philox block
 * (ev 0: launch {radius, angle, phi, tau}; each scatter {HG cosine, azimuth,
 * roulette, tau}; each Fresnel face {reflect test}). */
static void gen_packet(const orc_mc_desc *d, const void *grid, uint64_t pid, uint64_t seed, uint32_t stream,
                       double *jm, double *tal)
{
    const double hx = 2.0 * d->xmax / d->nx, hy = 2.0 * d->ymax / d->ny, hz = 2.0 * d->zmax / d->nz;
    const double BIG = 1.0e30;
    uint32_t ev = 0;
    double u[4];
    orc_philox_uniform4(seed, pid, stream, ev++, u);
    double r;
    if (d->source == ORC_SRC_DISK) r = sqrt(u[0] * (d->source_radius * d->source_radius));
    else r = d->source_radius * sqrt(-0.5 * log(u[0]));
    double theta = u[1] * TWOPI_R;
    double X = r * cos(theta) + d->xmax, Y = r * sin(theta) + d->ymax;
    double phi = TWOPI_R * u[2];
    double dir5[5] = {-1.0, 0.0, phi, cos(phi), sin(phi)};
    double w = 1.0;
    if (!(X >= 0.0 && X < 2.0 * d->xmax && Y >= 0.0 && Y < 2.0 * d->ymax)) {
        tal[ORC_T_MISSED] += w;
        return;
    }
    int ix = (int)(d->nx * X / (2.0 * d->xmax));
    int iy = (int)(d->ny * Y / (2.0 * d->ymax));
    if (ix > d->nx - 1) ix = d->nx - 1;
    if (iy > d->ny - 1) iy = d->ny - 1;
    int iz = d->nz - 1;
    double fx = X - ix * hx, fy = Y - iy * hy;
    double fz = hz - 1.e-8 * hz;
    medprops m;
    med_lookup(d, grid, ix, iy, iz, &m);
    if (d->fresnel) {
        double rsp = (d->n_ambient - m.n) / (d->n_ambient + m.n);
        rsp = rsp * rsp;
        tal[ORC_T_SPECULAR] += rsp;
        w = 1.0 - rsp;
    }
    double tau = -log(u[3]);
    double nx = dir5[1] * dir5[3], ny = dir5[1] * dir5[4], nz = dir5[0];
    double inx = 1.0 / nx, iny = 1.0 / ny, inz = 1.0 / nz;
    int64_t steps = 0;
    for (;;) {
        if (++steps > d->max_steps) {
            tal[ORC_T_OVERFLOW] += 1.0;
            break;
        }
        double ddx = nx > 0.0 ? (hx - fx) * inx : (nx < 0.0 ? -fx * inx : BIG);
        double ddy = ny > 0.0 ? (hy - fy) * iny : (ny < 0.0 ? -fy * iny : BIG);
        double ddz = nz > 0.0 ? (hz - fz) * inz : (nz < 0.0 ? -fz * inz : BIG);
        if (ddx < 0.0) ddx = 0.0;
        if (ddy < 0.0) ddy = 0.0;
        if (ddz < 0.0) ddz = 0.0;
        /* tie order of src/inttau2.f90:116-118: z over y over x */
        int ax = 2;
        double dw = ddz;
        if (ddy < dw) { dw = ddy; ax = 1; }
        if (ddx < dw) { dw = ddx; ax = 0; }
        double taucell = dw * m.mut;
        int64_t q = ix + (int64_t)d->nx * (iy + (int64_t)d->ny * iz);
        if (taucell < tau) {
            jm[q] += w * dw * m.mua;
            tau -= taucell;
            int nxt;
            if (ax == 0) {
                fy += ny * dw; fz += nz * dw;
                nxt = nx > 0.0 ? ix + 1 : ix - 1;
            } else if (ax == 1) {
                fx += nx * dw; fz += nz * dw;
                nxt = ny > 0.0 ? iy + 1 : iy - 1;
            } else {
                fx += nx * dw; fy += ny * dw;
                nxt = nz > 0.0 ? iz + 1 : iz - 1;
            }
            fx = fx < 0.0 ? 0.0 : (fx > hx ? hx : fx);
            fy = fy < 0.0 ? 0.0 : (fy > hy ? hy : fy);
            fz = fz < 0.0 ? 0.0 : (fz > hz ? hz : fz);
            int nax = ax == 0 ? d->nx : (ax == 1 ? d->ny : d->nz);
            double hn = ax == 0 ? hx : (ax == 1 ? hy : hz);
            double nc = ax == 0 ? nx : (ax == 1 ? ny : nz);
            if (nxt < 0 || nxt >= nax) {
                /* outer face: put the packet on it, then Fresnel or escape */
                if (ax == 0) fx = nc > 0.0 ? hn : 0.0;
                else if (ax == 1) fy = nc > 0.0 ? hn : 0.0;
                else fz = nc > 0.0 ? hn : 0.0;
                if (d->fresnel) {
                    orc_philox_uniform4(seed, pid, stream, ev++, u);
                    double R = orc_fresnel(m.n, d->n_ambient, fabs(nc));
                    if (u[0] < R) {
                        if (ax == 2) { dir5[0] = -dir5[0]; }
                        else if (ax == 0) {
                            dir5[3] = -dir5[3];
                            dir5[2] = PI_R - dir5[2];
                            if (dir5[2] < 0.) dir5[2] += TWOPI_R;
                        } else {
                            dir5[4] = -dir5[4];
                            dir5[2] = TWOPI_R - dir5[2];
                        }
                        nx = dir5[1] * dir5[3]; ny = dir5[1] * dir5[4]; nz = dir5[0];
                        inx = 1.0 / nx; iny = 1.0 / ny; inz = 1.0 / nz;
                        continue;
                    }
                }
                if (ax == 2) tal[nc > 0.0 ? ORC_T_REFLECTED : ORC_T_TRANSMITTED] += w;
                else tal[ORC_T_SIDE] += w;
                break;
            }
            if (ax == 0) { ix = nxt; fx = nx > 0.0 ? d->nudge : hx - d->nudge; }
            else if (ax == 1) { iy = nxt; fy = ny > 0.0 ? d->nudge : hy - d->nudge; }
            else { iz = nxt; fz = nz > 0.0 ? d->nudge : hz - d->nudge; }
            med_lookup(d, grid, ix, iy, iz, &m);
        } else {
            double dd = tau / m.mut;
            jm[q] += w * dd * m.mua;
            fx += nx * dd; fy += ny * dd; fz += nz * dd;
            fx = fx < 0.0 ? 0.0 : (fx > hx ? hx : fx);
            fy = fy < 0.0 ? 0.0 : (fy > hy ? hy : fy);
            fz = fz < 0.0 ? 0.0 : (fz > hz ? hz : fz);
            w *= m.albedo;
            if (w <= 0.0) break; /* pure absorber: the single flight of mcpolar.f90:166-169 */
            tal[ORC_T_SCATTERS] += 1.0;
            orc_philox_uniform4(seed, pid, stream, ev++, u);
            orc_stokes(m.g, m.g2, u[0], u[1], dir5);
            nx = dir5[1] * dir5[3]; ny = dir5[1] * dir5[4]; nz = dir5[0];
            inx = 1.0 / nx; iny = 1.0 / ny; inz = 1.0 / nz;
            if (d->roulette && w < d->roulette_w) {
                if (u[2] < 1.0 / d->roulette_m) {
                    tal[ORC_T_ROULETTE_NET] += w * (d->roulette_m - 1.0);
                    w *= d->roulette_m;
                } else {
                    tal[ORC_T_ROULETTE_NET] -= w;
                    break;
                }
            }
            tau = -log(u[3]);
        }
    }
    tal[ORC_T_STEPS] += (double)steps;
}

void orc_mc_transport(const orc_mc_desc *d, const void *grid, int64_t p0, int64_t n, uint64_t seed,
                      uint32_t stream, int nthreads, double *jmean, double *tallies)
{
    int T = nthr(nthreads);
    int64_t ni = (int64_t)d->nx * d->ny * d->nz;
    double *buf = NULL;
    if (T > 1) buf = (double *)calloc((size_t)T * (size_t)(ni + ORC_NTALLY), sizeof(double));
    if (!buf) {
        double tal[ORC_NTALLY] = {0};
        for (int64_t q = 0; q < n; ++q) gen_packet(d, grid, (uint64_t)(p0 + q), seed, stream, jmean, tal);
        double a = 0.0;
        for (int64_t q = 0; q < ni; ++q) a += jmean[q];
        for (int t = 0; t < ORC_NTALLY; ++t) tallies[t] += tal[t];
        tallies[ORC_T_ABSORBED] = a;
        return;
    }
#ifdef _OPENMP
#pragma omp parallel num_threads(T)
    {
        int t = omp_get_thread_num();
        double *jm = buf + (size_t)t * (size_t)(ni + ORC_NTALLY);
#pragma omp for schedule(dynamic, 64)
        for (int64_t q = 0; q < n; ++q) gen_packet(d, grid, (uint64_t)(p0 + q), seed, stream, jm, jm + ni);
    }
#endif
    for (int t = 0; t < T; ++t) {
        const double *jm = buf + (size_t)t * (size_t)(ni + ORC_NTALLY);
        for (int64_t q = 0; q < ni; ++q) jmean[q] += jm[q];
        for (int k = 0; k < ORC_NTALLY; ++k) tallies[k] += jm[ni + k];
    }
    double a = 0.0;
    for (int64_t q = 0; q < ni; ++q) a += jmean[q];
    tallies[ORC_T_ABSORBED] = a;
    free(buf);
}

/* ----------------------------------------------------- fused heat step -- */
double orc_stable_dt(const orc_heat_desc *h, double alpha_max)
{
    double s = 1.0 / (h->dx * h->dx) + 1.0 / (h->dy * h->dy) + 1.0 / (h->dz * h->dz);
    return 1.0 / (2.0 * h->opscale * alpha_max * s);
}

/* Face term of the reference stencil (src/3dFD.f90:119-132) with the operator
 * scale exposed: a = opscale * k_f / (rho_f c_f) / d^2 on each face. */
static inline double face_alpha(double kc, double kn, double rc, double rn, double cc, double cn)
{
    double kf = 0.5 * (kc + kn), rf = 0.5 * (rc + rn), cf = 0.5 * (cc + cn);
    return kf / (rf * cf);
}

int64_t orc_fused_step(const orc_heat_desc *h, double P, double t_new, const double *T, double *Tn,
                       const double *k, const double *rho, const double *c, double *J, double *Q,
                       double *omega, double *thres, uint8_t *mat, int nthreads)
{
    const int nx = h->nx, ny = h->ny, nz = h->nz;
    const int64_t sx = 1, sy = nx, sz = (int64_t)nx * ny, ni = sz * nz;
    const double id2[3] = {1.0 / (h->dx * h->dx), 1.0 / (h->dy * h->dy), 1.0 / (h->dz * h->dz)};
    const double dd[3] = {h->dx, h->dy, h->dz};
    int T_ = nthr(nthreads);
    (void)T_;
    int64_t nabl = 0;
#ifdef _OPENMP
#pragma omp parallel for num_threads(T_) schedule(static) reduction(+ : nabl)
#endif
    for (int iz = 0; iz < nz; ++iz)
        for (int iy = 0; iy < ny; ++iy)
            for (int ix = 0; ix < nx; ++ix) {
                int64_t v = ix + sy * iy + sz * iz;
                double T0 = T[v], kv = k[v], rv = rho[v], cv = c[v];
                int idx[3] = {ix, iy, iz};
                int nn[3] = {nx, ny, nz};
                int64_t st[3] = {sx, sy, sz};
                double lap = 0.0;
                for (int a = 0; a < 3; ++a) {
                    double Tm, Tp, am, ap;
                    if (idx[a] > 0) {
                        int64_t m = v - st[a];
                        Tm = T[m];
                        am = face_alpha(kv, k[m], rv, rho[m], cv, c[m]);
                    } else {
                        int f = 2 * a;
                        Tm = h->bc_type[f] == ORC_BC_ROBIN ? T0 - (h->bc_h[f] * dd[a] / kv) * (T0 - h->bc_Tamb[f])
                                                          : h->bc_T[f];
                        am = kv / (rv * cv);
                    }
                    if (idx[a] < nn[a] - 1) {
                        int64_t pn = v + st[a];
                        Tp = T[pn];
                        ap = face_alpha(kv, k[pn], rv, rho[pn], cv, c[pn]);
                    } else {
                        int f = 2 * a + 1;
                        Tp = h->bc_type[f] == ORC_BC_ROBIN ? T0 - (h->bc_h[f] * dd[a] / kv) * (T0 - h->bc_Tamb[f])
                                                          : h->bc_T[f];
                        ap = kv / (rv * cv);
                    }
                    double A = h->opscale * am * id2[a];
                    double D = h->opscale * ap * id2[a];
                    lap += A * (Tm - T0) + D * (Tp - T0);
                }
                double dT = h->dt * lap;
                double src = P * J[v] * h->dt / (rv * cv);
                double Tnew;
                double qv = h->lw * rv * h->vvox;
                if (h->boil && T0 >= h->T_boil && Q[v] < qv) {
                    double E = (P * J[v] * h->dt + rv * cv * dT) * h->vvox;
                    if (E > 0.0) {
                        double qn = Q[v] + E;
                        Q[v] = qn < qv ? qn : qv;
                        Tnew = h->T_boil;
                    } else {
                        Tnew = T0 + (dT + src);
                    }
                } else {
                    Tnew = T0 + (dT + src);
                }
                Tn[v] = Tnew;
                if (h->arrhenius && Tnew >= h->T_lo && Tnew < h->T_hi) {
                    double o = omega[v];
                    double on = o + h->dt * exp(h->lnA - h->Ea / (h->Rgas * Tnew));
                    omega[v] = on;
                    for (int t = 0; t < 3; ++t)
                        if (o < h->thr[t] && on >= h->thr[t]) thres[v + t * ni] = t_new;
                }
                if (Tnew >= h->T_abl && mat[v] != 0) {
                    mat[v] = 0; /* optics -> air; the source of this voxel stops */
                    J[v] = 0.0;
                    nabl += 1;
                }
            }
    return nabl;
}

/* src/3dFD.f90:330-349: do k / do j / do i, summ of the six neighbours,
 * in place (the backward neighbours are already updated). */
int64_t orc_isolate(int nx, int ny, int nz, uint8_t *mat, double *J)
{
    const int64_t sy = nx, sz = (int64_t)nx * ny;
    int64_t n = 0;
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                const int64_t v = i + sy * j + sz * k;
                if (mat[v] == 0) continue;
                int summ = 0;
                summ += k + 1 < nz ? mat[v + sz] : 0;
                summ += j + 1 < ny ? mat[v + sy] : 0;
                summ += i + 1 < nx ? mat[v + 1] : 0;
                summ += k > 0 ? mat[v - sz] : 0;
                summ += j > 0 ? mat[v - sy] : 0;
                summ += i > 0 ? mat[v - 1] : 0;
                if (summ == 0) {
                    mat[v] = 0;
                    J[v] = 0.0;
                    n += 1;
                }
            }
    return n;
}
