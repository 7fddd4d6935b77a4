/*
 * tam_oracle.h -- CPU oracle for the two hot paths of Tissue-Ablation-MC.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C FP64 restatement of the
 * reference Fortran (lewisfish/Tissue-Ablation-MC) that the tests check the
 * CUDA library against.  Only tests/, __graft_entry__.smoke() and the CPU legs of
 * bench.py may load it; the product library never links or calls it.
 *
 * Parity status: parity unpinned.  The reference cannot be compiled (no
 * Fortran compiler or MPI exists on either machine) and ships no tests,
 * fixtures or golden vectors, so no reference output exists to pin against.
 * The oracle is instead checked by analytic known-answer tests derived from
 * the reference's own equations (Beer-Lambert depth profile of the pure
 * absorber, the discrete eigen-decay of the reference's halved diffusion
 * operator, constant-temperature Arrhenius integrals and threshold chain, HG
 * mean cosine, normal-incidence Fresnel, energy balance) and by regression
 * vectors generated from it and committed under tests/golden/.
 *
 * Two semantic modes:
 *   (R) reference mode -- statement-by-statement restatement of the compiled
 *       Fortran path (pure absorber, single flight, Dirichlet faces, halved
 *       operator, water-content property model).  Functions orc_ref_*.
 *   (C) config mode -- the physics the benchmark configurations ask for
 *       (HG scattering with stokes.f90 semantics, Fresnel faces, Russian
 *       roulette, Gaussian beam, Robin top face, material table, non-cubic
 *       grids, fused FP64 heat step).  Functions orc_mc_* / orc_fused_*.
 *
 * The random numbers are NOT the reference's ran2 (src/ran2.f, Numerical
 * Recipes); both the oracle and the GPU draw from Philox4x32-10 (Salmon et
 * al., SC'11) with the per-packet event counter layout described in
 * orc_philox_uniform4(), so oracle and GPU consume identical streams.
 */
#ifndef TAM_ORACLE_H
#define TAM_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- RNG --- */

/* Philox4x32-10 block function.  ctr[4], key[2] -> out[4]. */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

/* Four FP64 uniforms in (0,1) for event `ev` of packet `pid` of stream
 * `stream` under 64-bit `seed`: counter = {ev, pid_lo, pid_hi, stream},
 * key = {seed_lo, seed_hi}, u = (x + 0.5) * 2^-32. */
void orc_philox_uniform4(uint64_t seed, uint64_t pid, uint32_t stream, uint32_t ev, double u[4]);

/* ---------------------------------------------------- reference mode --- */

enum { ORC_PULSE_GAUSSIAN = 0, ORC_PULSE_TOPHAT = 1, ORC_PULSE_TRIANGULAR = 2 };

/* The 14 fields of res/input.params (read at src/mcpolar.f90:79-94) plus
 * the compile-time grid (src/constants.f90:12). */
typedef struct {
    int64_t nphotons;
    double xmax, ymax, zmax;      /* half-widths, cm */
    double n1, n2;
    double total_time;            /* s */
    int32_t loops;
    double repetition_rate_1;     /* s (compared against an elapsed time) */
    double power;                 /* W */
    double energy_per_pixel;      /* mJ */
    double ablate_temp;           /* deg C */
    int32_t pulses_to_do;
    int32_t pulse_type;           /* ORC_PULSE_* */
    int32_t nx, ny, nz;           /* nxg, nyg, nzg */
    int32_t numproc;              /* ranks in the normalisation (mcpolar.f90:174) */
} orc_ref_params;

/* Module state of the reference (iarray, opt_prop, Heat, thermalConstants).
 * Array layouts are Fortran column-major, x fastest:
 *   halo arrays  (0:n+1)^3 : idx = i + (nx+2)*(j + (ny+2)*k)
 *   interior     (1:n)^3   : idx = (i-1) + nx*((j-1) + ny*(k-1))
 *   thres        interior x 3 (last index slowest)                       */
typedef struct {
    orc_ref_params p;
    /* opt_prop (src/opt_prop.f90:5, src/ch_opt.f90:15-22) */
    double hgg, g2, mua, mus, kappa_opt, albedo, mu_water, mu_protein;
    double delta;                 /* src/mcpolar.f90:112 */
    /* module Heat scalars (src/3dFD.f90:7-12) */
    double delt, dx, dy, dz, volumeVoxel, massVoxel, QVapor;
    double pulseLength, realPulseLength;
    double time, pulseCount, repetitionCount, laserOn;
    int32_t laser_flag, pulseFlag, pulsesDone, loops_left, counter;
    double skinDensityInit;
    int32_t error;                /* nonzero: an `error stop`/`mpi_abort` site fired */
    /* iarray */
    double *xface, *yface, *zface; /* 1-based, n+1 entries used ([0] unused) */
    double *rhokap;               /* halo */
    double *jmean, *jmeanGLOBAL;  /* interior */
    double *temp;                 /* halo */
    double *tissue, *thres;       /* interior, interior x 3 */
    /* module Heat arrays */
    double *kappa, *density, *heatcap, *coeff, *alpha; /* halo */
    double *Q, *water;            /* interior */
} orc_ref_state;

/* alloc_array + zarray + init_opt1 + gridset + temp init + initThermalCoeff +
 * the total_time override: everything src/mcpolar.f90:55-140 does before the
 * outer loop.  Returns NULL on allocation failure or bad pulse type. */
orc_ref_state *orc_ref_create(const orc_ref_params *p);
void orc_ref_free(orc_ref_state *s);

/* sourcephCO2 + tauint1 for packets [p0, p0+n) accumulated into s->jmean
 * (src/mcpolar.f90:151-170).  Statement-by-statement arithmetic of
 * src/sourceph.f90:7-49 and src/inttau2.f90:7-239 (find() bisection,
 * exact-equality wall test, delta snapping). */
void orc_ref_photons(orc_ref_state *s, int64_t p0, int64_t n, uint64_t seed, uint32_t stream, int nthreads);
/* jmeanGLOBAL = jmean * (getPwr()/81) / (nphotons*numproc*Vvox)  (mcpolar.f90:173-174) */
void orc_ref_normalise(orc_ref_state *s);
/* getPwr at the current module time (src/3dFD.f90:365-421); may mutate pulseFlag. */
double orc_ref_get_pwr(orc_ref_state *s);
/* heat_sim_3D, single rank (src/3dFD.f90:21-230). Returns 0 or an error code. */
int orc_ref_heat_sim(orc_ref_state *s, int nthreads);
/* Arrhenius (src/3dFD.f90:424-466). */
void orc_ref_arrhenius(orc_ref_state *s);
/* setupThermalCoeff (src/3dFD.f90:312-361), sequential sweep exactly as written. */
void orc_ref_setup_thermal(orc_ref_state *s);
/* One iteration of the outer do-while loop (src/mcpolar.f90:148-186). */
int orc_ref_outer_iteration(orc_ref_state *s, uint64_t seed, int nthreads);
/* Runs the outer loop while time <= total_time, at most max_iters iterations
 * (<=0: unbounded).  Returns the iteration count or a negative error. */
int64_t orc_ref_run(orc_ref_state *s, uint64_t seed, int64_t max_iters, int nthreads);
/* tissue(rhokap <= 0.1) = -1 (src/mcpolar.f90:196-204). */
void orc_ref_finalize(orc_ref_state *s);

/* Thermal property functions (src/thermalConst_mod.f90:11-87). */
double orc_air_thermal_cond(double T);
double orc_air_density(double T);
double orc_skin_density(double w);
double orc_skin_heat_cap(double w);
double orc_skin_thermal_cond(double w, double rho);
double orc_water_content(double Q, double w, double QVapor);

/* HG deflection with the exact arithmetic of src/stokes.f90:6-153.
 * dir = {cost, sint, phi, cosp, sinp} updated in place; u0 feeds the HG
 * cosine (stokes.f90:48 / :24), u1 the azimuth (stokes.f90:64 / :32). */
void orc_stokes(double hgg, double g2, double u0, double u1, double dir[5]);

/* ------------------------------------------------------- config mode --- */

#define ORC_MAX_MAT 16
enum { ORC_SRC_DISK = 0, ORC_SRC_GAUSSIAN = 1 };
enum { ORC_MED_RHOKAP = 0, ORC_MED_MATERIAL = 1 };
enum { ORC_T_ABSORBED = 0, ORC_T_SPECULAR, ORC_T_REFLECTED, ORC_T_TRANSMITTED, ORC_T_SIDE,
       ORC_T_ROULETTE_NET, ORC_T_MISSED, ORC_T_STEPS, ORC_T_SCATTERS, ORC_T_OVERFLOW, ORC_NTALLY };

typedef struct {
    double mua, mus, g, n;        /* /cm, /cm, -, - */
} orc_optmat;

/* Generic transport description shared with the GPU kernel. */
typedef struct {
    int32_t nx, ny, nz;
    double xmax, ymax, zmax;      /* half-widths, cm */
    int32_t medium;               /* ORC_MED_* */
    int32_t nmat;
    orc_optmat mat[ORC_MAX_MAT];  /* material 0 is the ablated / air entry */
    double n_ambient;
    int32_t source;               /* ORC_SRC_* */
    double source_radius;         /* disk radius or Gaussian 1/e^2 radius, cm */
    int32_t fresnel;              /* specular entry + Fresnel faces */
    int32_t roulette;
    double roulette_w, roulette_m;
    double rhokap_n;              /* refractive index used with the rhokap medium */
    int64_t max_steps;            /* per-packet loop cap (error if exceeded) */
    double nudge;                 /* offset past a crossed face: the reference's delta
                                     (src/mcpolar.f90:112, src/inttau2.f90:142-166), 0 in config mode */
} orc_mc_desc;

/* Transport of packets [p0, p0+n): jmean (interior, packet units: sum of
 * w*d*mua) and tallies[ORC_NTALLY] are accumulated.  For ORC_MED_RHOKAP,
 * `grid` points to a halo (nx+2)(ny+2)(nz+2) double array (mut = mua =
 * rhokap, albedo 0); for ORC_MED_MATERIAL to nx*ny*nz uint8 ids. */
void orc_mc_transport(const orc_mc_desc *d, const void *grid, int64_t p0, int64_t n,
                      uint64_t seed, uint32_t stream, int nthreads, double *jmean, double *tallies);

/* Unpolarised Fresnel reflectance, n1 -> n2 at incidence cosine cosi. */
double orc_fresnel(double n1, double n2, double cosi);

enum { ORC_BC_DIRICHLET = 0, ORC_BC_ROBIN = 1 };

/* Fused config-mode heat step description (stencil + boiling clamp +
 * Arrhenius + ablation), shared with the GPU fused kernel. */
typedef struct {
    int32_t nx, ny, nz;
    double dx, dy, dz;            /* m */
    double opscale;               /* 1.0 full operator; 0.5 reproduces the reference's halving */
    double dt;                    /* s */
    double vvox;                  /* m^3 */
    int32_t boil;
    double T_boil, lw;
    double T_abl;                 /* K */
    int32_t arrhenius;
    double lnA, Ea, Rgas, T_lo, T_hi;
    double thr[3];
    int32_t bc_type[6];           /* faces x-, x+, y-, y+, z-, z+ */
    double bc_T[6], bc_h[6], bc_Tamb[6];
} orc_heat_desc;

/* One fused step over interior arrays (x fastest).  Reads T, writes Tn.
 * P multiplies the source J (W/m^3 per unit).  t_new is the time stamp
 * recorded on a threshold crossing.  Newly ablated voxels (Tn >= T_abl,
 * mat != 0) get mat = 0 and J = 0 (no other voxel reads them); their count is returned. */
int64_t orc_fused_step(const orc_heat_desc *h, double P, double t_new,
                       const double *T, double *Tn, const double *k, const double *rho,
                       const double *c, double *J, double *Q, double *omega, double *thres,
                       uint8_t *mat, int nthreads);

/* The isolation rule of src/3dFD.f90:347-349 on a config-mode material grid
 * (u8, x fastest): the reference's sequential sweep (k, j, i) with its
 * in-place updates, where a voxel that is not air (id != 0) and whose six
 * neighbours are air -- outside the grid counting as air, as the
 * reference's zero halo -- becomes air and its source J goes to zero.
 * Returns the number of voxels turned to air. */
int64_t orc_isolate(int nx, int ny, int nz, uint8_t *mat, double *J);

/* Stability-limited step of the config-mode operator: 1/(2 opscale amax sum 1/d^2). */
double orc_stable_dt(const orc_heat_desc *h, double alpha_max);

#ifdef __cplusplus
}
#endif
#endif
