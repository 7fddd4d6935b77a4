/*
 * tam.h -- C ABI of the GB300-native hot paths of Tissue-Ablation-MC.
 *
 * The reference (lewisfish/Tissue-Ablation-MC, Fortran + MPI) has no plugin or
 * FFI: its "API" is the set of Fortran subroutines called from the driver
 * loop in src/mcpolar.f90:148-186, communicating through module globals.  A
 * per-photon FFI call is not viable, so this ABI replaces whole blocks of that
 * loop:
 *   - the photon loop + MPI_Allreduce + normalisation (src/mcpolar.f90:151-174)
 *     -> tam_mc_pass
 *   - heat_sim_3D (src/mcpolar.f90:178)            -> tam_heat_steps
 *   - Arrhenius (src/mcpolar.f90:180)              -> tam_arrhenius
 *   - setupThermalCoeff (src/mcpolar.f90:182)      -> tam_update_props
 *   - one whole outer iteration / the whole loop   -> tam_step_coupled / tam_run
 *
 * Conventions
 *   - Plain C types only; every call returns an int status (TAM_OK == 0);
 *     tam_last_error() gives a one-line message.  Nothing aborts the process:
 *     the reference's `error stop` / `mpi_abort` sites become status codes.
 *   - Arrays exchanged with the host use the reference layout: FP64,
 *     Fortran column-major (x fastest), with the reference's halo where the
 *     reference allocates one (start index 0, src/subs.f90:62-73,
 *     src/3dFD.f90:254-260).
 *   - A context owns its device state, which stays resident across calls.
 *     A context is not thread-safe; use one per host thread.  All work of a
 *     context is issued on one CUDA stream (its own, or one set with
 *     tam_set_stream) and each hot call returns after that work completes.
 *   - No CPU fallback: tam_create fails with TAM_E_NODEV without a GPU.
 */
#ifndef TAM_H
#define TAM_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TAM_ABI_VERSION 2

/* The library's context (opaque).  Declared here, at file scope, so that
 * every prototype below names this one type when the header is compiled as
 * C (a struct first named inside a parameter list would be a new type). */
struct tam_ctx;

/* ---- status codes ---- */
enum tam_status {
    TAM_OK = 0,
    TAM_E_INVALID = 1,   /* bad argument or parameter value */
    TAM_E_CUDA = 2,      /* CUDA runtime error */
    TAM_E_NOMEM = 3,     /* device allocation failed */
    TAM_E_IO = 4,        /* file could not be opened / written */
    TAM_E_PARSE = 5,     /* input.params could not be parsed */
    TAM_E_STATE = 6,     /* call not valid in this mode / state */
    TAM_E_DEVICE = 7,    /* a kernel raised its error word (see tam_device_errors) */
    TAM_E_NODEV = 8      /* no CUDA device */
};

enum tam_mode { TAM_MODE_REFERENCE = 0, TAM_MODE_CONFIG = 1 };
enum tam_precision { TAM_FP64 = 0, TAM_FP32 = 1 };
enum tam_pulse { TAM_PULSE_GAUSSIAN = 0, TAM_PULSE_TOPHAT = 1, TAM_PULSE_TRIANGULAR = 2 };
enum tam_source { TAM_SRC_DISK = 0, TAM_SRC_GAUSSIAN = 1 };
enum tam_bc { TAM_BC_DIRICHLET = 0, TAM_BC_ROBIN = 1 };

/* Device error-word bits returned by tam_device_errors. */
#define TAM_DEVERR_STEP_CAP 0x1u  /* a packet hit its step cap and was killed */
#define TAM_DEVERR_NAN 0x2u       /* NaN direction or temperature */
#define TAM_DEVERR_NEG_T 0x4u     /* negative kelvin (src/3dFD.f90:179-182) */

/*
 * Run parameters.  The first block is res/input.params in file order, as read
 * by src/mcpolar.f90:79-94.  The grid is compile-time in the reference
 * (src/constants.f90:12) and a run-time field here; numproc reproduces the
 * nphotons*numproc divisor of src/mcpolar.f90:174.
 */
typedef struct tam_params {
    int64_t nphotons;            /* packets per MC pass */
    double xmax, ymax, zmax;     /* half-widths, cm */
    double n1, n2;               /* refractive indices (ambient, tissue) */
    double total_time;           /* s */
    int32_t loops;               /* heat steps per outer iteration */
    double repetition_rate_1;    /* s, pulse repetition period */
    double power;                /* W */
    double energy_per_pixel;     /* mJ */
    double ablate_temp;          /* deg C */
    int32_t pulses_to_do;
    int32_t pulse_type;          /* enum tam_pulse */
    int32_t nxg, nyg, nzg;       /* grid */
    int32_t numproc;             /* normalisation divisor, >= 1 */
    int32_t mode;                /* enum tam_mode */
    int32_t precision;           /* enum tam_precision: transport and heat step (reference mode:
                                    FP32 stencil, increments added to FP64 temperatures) */
    int32_t device;              /* CUDA device ordinal */
} tam_params;

#define TAM_MAX_MATERIALS 16

/* Optical + thermal properties of one material.  Material 0 is the
 * ablated state ("air"): its optics are used for ablated voxels. */
typedef struct tam_material {
    double mua, mus, g, n;       /* /cm, /cm, HG anisotropy, refractive index */
    double k, rho, c;            /* W/m/K, kg/m^3, J/kg/K */
} tam_material;

/*
 * Config-mode extension (no slot in the reference's input.params): material
 * table, beam, boundaries, Arrhenius constants.  Ignored in reference mode.
 */
typedef struct tam_config {
    int32_t nmat;
    tam_material mat[TAM_MAX_MATERIALS];
    double n_ambient;
    int32_t source;              /* enum tam_source */
    double source_radius;        /* disk radius or Gaussian 1/e^2 radius, cm */
    int32_t fresnel;             /* specular entry + Fresnel at the outer faces */
    int32_t roulette;
    double roulette_w, roulette_m;
    double T0;                   /* initial tissue temperature, K */
    int32_t bc_type[6];          /* faces x-, x+, y-, y+, z- (bottom), z+ (top, beam side) */
    double bc_T[6], bc_h[6], bc_Tamb[6];
    double dt_factor;            /* dt = dt_factor * stability limit */
    double dt;                   /* if > 0, overrides dt_factor */
    double opscale;              /* 1 = physical operator */
    int32_t boil;
    double T_boil, lw;
    double T_abl;                /* K */
    int32_t arrhenius;
    double A, Ea, Rgas, T_lo, T_hi;
    double thr[3];
    double retrace_fraction;     /* re-run MC when newly ablated > fraction of grid; <=0 never */
    int32_t retrace_check;       /* heat steps between re-trace checks, counted across calls
                                  * (0: at the end of every heat-step call) */
    int64_t max_steps;           /* per-packet loop cap */
    int32_t isolation;           /* 1: after every heat step a tissue voxel whose six neighbours are all air
                                  * (outside the grid counts as air) turns to air, the rule of
                                  * src/3dFD.f90:347-349; 0 (default): no such rule */
} tam_config;

/* Mutable module scalars of the reference (module Heat, src/3dFD.f90:7-12). */
typedef struct tam_state {
    double time, delt, total_time, pulse_count, repetition_count, laser_on;
    double pulse_length, real_pulse_length, volume_voxel, mass_voxel, qvapor;
    double dx, dy, dz;
    int32_t laser_flag, pulse_flag, pulses_done, counter;
    int64_t n_ablated;           /* config mode: voxels ablated so far */
    int64_t mc_passes;
} tam_state;

/* Fields for tam_upload / tam_download / tam_field_bytes. */
enum tam_field {
    TAM_F_TEMP = 0,        /* (0:nx+1,0:ny+1,0:nz+1) K            src/iarray.f90:10 */
    TAM_F_RHOKAP = 1,      /* (0:nx+1,...) /cm, halo 0             src/iarray.f90:9 */
    TAM_F_JMEAN = 2,       /* (1:nx,1:ny,1:nz) packet units        src/iarray.f90:10 */
    TAM_F_JMEAN_GLOBAL = 3,/* (1:nx,...) W/m^3 (config: per W)     src/mcpolar.f90:174 */
    TAM_F_TISSUE = 4,      /* (1:nx,...) Omega                     src/3dFD.f90:451 */
    TAM_F_THRESTIME = 5,   /* (1:nx,...,3) s                       src/3dFD.f90:455-461 */
    TAM_F_KAPPA = 6,       /* (0:nx+1,...) W/m/K                   src/3dFD.f90:256 */
    TAM_F_DENSITY = 7,     /* (0:nx+1,...) kg/m^3 */
    TAM_F_HEATCAP = 8,     /* (0:nx+1,...) J/kg/K */
    TAM_F_COEFF = 9,       /* (0:nx+1,...) reference mode only */
    TAM_F_ALPHA = 10,      /* (0:nx+1,...) reference mode only */
    TAM_F_Q = 11,          /* (1:nx,...) J latent heat */
    TAM_F_WATER = 12,      /* (1:nx,...) reference mode only */
    TAM_F_MATERIAL = 13,   /* (1:nx,...) uint8 material id, config mode only */
    TAM_NFIELDS = 14
};

/* Library identification. */
const char *tam_version(void);
int tam_abi_version(void);
/* sizeof the ABI structs, for FFI layout checks: 0 tam_params, 1 tam_config,
 * 2 tam_state, 3 tam_material; -1 otherwise. */
int64_t tam_struct_size(int32_t which);

/* The shipped res/input.params values on the 80^3 grid, reference mode, FP64. */
int tam_params_default(tam_params *p);
/* Config-mode defaults (homogeneous tissue, Gaussian beam, Robin top face). */
int tam_config_default(tam_config *c);

/*
 * Parse res/input.params with Fortran list-directed semantics: one value per
 * line in the order of src/mcpolar.f90:79-94; the rest of each line is
 * ignored; ',' '/' and blanks end a value; 'd'/'D' exponents accepted.
 * Fields not in the file (grid, mode, ...) are left untouched.
 */
int tam_read_input_params(const char *path, tam_params *p);
/*
 * Parse a config-mode extension file (the parameters input.params has no slot
 * for; e.g. res/tissue.params beside it) into *c, which holds the values the
 * file leaves out (start from tam_config_default).  One setting per line,
 * '#' starts a comment:
 *   nmat N
 *   material I mua mus g n k rho c   (/cm, /cm, -, -, W/m/K, kg/m^3, J/kg/K;
 *                                      raises nmat to I + 1 when needed)
 *   source gaussian|disk   source_radius R   n_ambient N
 *   fresnel 0|1   roulette 0|1   roulette_w W   roulette_m M   max_steps S
 *   bc FACE dirichlet T=K   |   bc FACE robin h=H Tamb=K
 *                                     (FACE: x- x+ y- y+ z- z+; z+ is the beam side)
 *   T0 K   dt_factor F   dt S   opscale F   boil 0|1   T_boil K   lw J/kg
 *   T_abl K   arrhenius 0|1   A 1/s   Ea J/mol   Rgas J/mol/K   T_lo K
 *   T_hi K   thr O1 O2 O3   retrace_fraction F   retrace_check N
 *   isolation 0|1
 * TAM_E_IO if the file cannot be opened; TAM_E_PARSE (with "path:line: ..."
 * from tam_last_error(NULL)) for an unknown key or a malformed value, in
 * which case *c is left unchanged.
 */
int tam_read_config(const char *path, tam_config *c);

/*
 * Create a context: allocates the device state and runs the initialisation
 * of src/mcpolar.f90:55-140 (alloc_array, zarray, init_opt1, gridset,
 * temperature init, initThermalCoeff, total_time override) in reference
 * mode, or the material/thermal set-up in config mode (cfg != NULL).
 */
int tam_create(const tam_params *p, const tam_config *cfg, struct tam_ctx **out);
int tam_destroy(struct tam_ctx *ctx);
/* Last error message of ctx (or of this thread when ctx is NULL). */
const char *tam_last_error(const struct tam_ctx *ctx);
/* Issue all further work of ctx on the given cudaStream_t (NULL: own stream). */
int tam_set_stream(struct tam_ctx *ctx, void *cuda_stream);
/* Bits of the device error word accumulated since creation. */
int tam_device_errors(struct tam_ctx *ctx, uint32_t *bits);

/* Re-run the set-up subroutines (tam_create already ran them).
 *   init_opt1 (src/ch_opt.f90:7-25), gridset (src/gridset.f90:6-46),
 *   initThermalCoeff (src/3dFD.f90:233-309). */
int tam_init_opt(struct tam_ctx *ctx);
int tam_gridset(struct tam_ctx *ctx, double xmax, double ymax, double zmax);
int tam_init_thermal(struct tam_ctx *ctx, double *delt);

/* Host <-> device copies of one field in the reference layout. */
int tam_field_bytes(struct tam_ctx *ctx, int field, int64_t *nbytes);
int tam_upload(struct tam_ctx *ctx, int field, const void *host, int64_t nbytes);
int tam_download(struct tam_ctx *ctx, int field, void *host, int64_t nbytes);

/*
 * One MC pass of nphotons packets (packet ids 0..nphotons-1, Philox stream
 * `stream` under `seed`): sourcephCO2 + tauint1 (+ stokes in config mode)
 * for every packet (src/mcpolar.f90:151-170), the tally reduction
 * (src/mcpolar.f90:173) and the normalisation (src/mcpolar.f90:174):
 *   reference mode: jmeanGLOBAL = jmean * (getPwr()/81)/(nphotons*numproc*Vvox)
 *   config mode:    jmeanGLOBAL = jmean / (nphotons * Vvox)   [W/m^3 per W]
 * jmean_out (nullable) receives jmeanGLOBAL, nx*ny*nz doubles.
 */
int tam_mc_pass(struct tam_ctx *ctx, int64_t nphotons, uint64_t seed, uint32_t stream, double *jmean_out);

/*
 * Heat steps.  Reference mode: heat_sim_3D with `nsteps` loops
 * (src/3dFD.f90:21-230), including the pulse state machine.  Config mode:
 * nsteps fused steps (stencil + latent-heat clamp + Arrhenius + ablation).
 * temp_out (nullable) receives the (nx+2)(ny+2)(nz+2) temperature.
 */
int tam_heat_steps(struct tam_ctx *ctx, int32_t nsteps, double *temp_out);
/* Arrhenius (src/3dFD.f90:424-466), reference mode. */
int tam_arrhenius(struct tam_ctx *ctx);
/* setupThermalCoeff (src/3dFD.f90:312-361), reference mode. */
int tam_update_props(struct tam_ctx *ctx, double ablate_temp);
/* n iterations of the outer loop of src/mcpolar.f90:148-186.  The device
 * error word is checked every 64 iterations and after the last, so the loop
 * runs ahead of the device in between. */
int tam_step_coupled(struct tam_ctx *ctx, int32_t n, uint64_t seed);
/* The whole outer loop while time <= total_time (at most max_iters, <=0 no
 * cap), with the same error checks. */
int tam_run(struct tam_ctx *ctx, uint64_t seed, int64_t max_iters, int64_t *iters);
/* tissue(rhokap <= 0.1) = -1 (src/mcpolar.f90:196-204). */
int tam_finalize(struct tam_ctx *ctx);

/* Tallies of the last MC pass, as fractions of launched packets.
 * The reference never records escapes (src/inttau2.f90:58-61). */
int tam_get_tallies(struct tam_ctx *ctx, double *absorbed, double *reflected, double *transmitted);
/* All tally slots of the last pass: absorbed, specular, reflected,
 * transmitted, side, roulette_net, missed, voxel_steps, scatters, overflow. */
int tam_get_tallies_ex(struct tam_ctx *ctx, double *out, int32_t n);
int tam_get_state(struct tam_ctx *ctx, tam_state *st);

/* Device time of the last hot calls, from CUDA events recorded on the
 * context's stream: the transport kernel of the last MC pass (for a batched
 * pass, the batched launch that carried it), and the span of the last run of
 * heat steps from its first to its last kernel, with the number of heat
 * kernels it launched (graph replays count their kernels).  In the coupled
 * loops these are the last iteration's pass and steps. */
int tam_get_timing(struct tam_ctx *ctx, double *transport_ms, double *heat_ms, int64_t *heat_launches);
/* Kernel tuning knobs (no reference counterpart; defaults are tuned for
 * GB300).  Keys: "transport.scat_min" (lanes of a warp that wait at an
 * interaction before the warp scatters, 1..32), "transport.tally32" (FP32
 * config-mode transport: -1 (default) deposits into an FP32 tally flushed
 * into the FP64 jmean when the FP64 tally exceeds 256 MB, 0 never, 1 always),
 * "transport.tally32_chunk" (packets per flush, default 16777216),
 * "transport.tally32_box" (cells of the FP32 tally at most, default 25165824
 * = 96 MB: larger grids get a box of that many cells centred on the beam axis
 * and reaching down from the top face, whose deposits are tallied in FP32;
 * deposits outside it go to the FP64 jmean directly; FP64 contexts use the
 * FP32 tally only with "transport.tally32" 1), "transport.bricks" (config-mode
 * transport on a heterogeneous grid: -1 (default) looks the cells' materials
 * up through a table of 8 x 8 x 8 bricks -- the one material of a brick, or
 * the grid itself inside mixed bricks -- for grids of 2^25 voxels or more, 0
 * never, 1 always; same walks either way), "heat.zchunk" (z planes per
 * thread column of the fused step, 0 = automatic; on a grid of several
 * thermal classes a change rebuilds the slab form's lists of one-class and
 * mixed blocks and synchronises the context's stream), "heat.tma" (1: stage the
 * FP32 fused step's planes with TMA where the row pitch allows, 0: cp.async),
 * "heat.cls" (1: while the thermal properties are those of the material
 * classes, look the face coefficients up per class pair instead of reading
 * per-voxel coefficient arrays; 0: always read the arrays; with TMA off or
 * rows whose pitch TMA cannot take (nx not a multiple of 4) the class-table
 * step stages its planes with cp.async, two voxels per thread),
 * "heat.slab" (class-table step with TMA: 1 (default) runs the slab form --
 * tiles of 32 x 8 voxels, two x-adjacent voxels per thread, one block
 * barrier per plane, boundary faces as ghost neighbours, boiling, damage and
 * ablation done for the listed voxels after the planes; 0 runs the form
 * chosen by "heat.cls_rows"),
 * "heat.cls_rows" (class-table step without the slab form: 0 = two
 * x-adjacent voxels per thread; 1 or 2 = that many voxel rows per thread),
 * "heat.graph" (config mode: 1 (default) replays chunks of 16 heat steps from
 * CUDA graphs when no step but a chunk's last needs the host (re-trace check,
 * source switching on); 0 launches every step),
 * "heat.arrhenius_fp64" (FP32 form: 1 evaluates the Arrhenius exponent
 * ln A - Ea/RT in FP64, 0 (default) in float-float arithmetic, ~44 bits),
 * "batch.zchunk" (batched heat steps, read from the first context of the
 * batch: z planes per work item; 0 (default) uses each instance's
 * "heat.zchunk" if set, else 32; the slab form's items hold at most 128
 * planes (batch.staged 4) or 32 (3)),
 * "batch.staged" (batched heat steps, read from the first context of the
 * batch: 4 (default) and 3 are the slab form -- each staged row the 16-byte
 * chunks that cover it, copied by all threads with cp.async, voxel pairs,
 * boundary faces as ghost neighbours; 4 launches one block per work item and
 * step and handles the voxels needing rare work (boiling, damage window,
 * ablation) in a second kernel over the step's list of them, 3 runs a chunk
 * of steps in one cooperative launch and handles them after each item's
 * planes; 2 stages each tile's planes in shared memory with 4-byte cp.async
 * copies and updates two x-adjacent voxels per thread, 1 the same with one
 * voxel per thread, 0 reads neighbours with cached global loads),
 * "batch.streams" (batched heat steps, read from the first context: 1 runs
 * each instance's own single-context steps on its own stream, issued
 * round-robin in chunks of 256 steps so the instances overlap, instead of
 * the one cooperative launch of 0, the default). */
int tam_set_tuning(struct tam_ctx *ctx, const char *key, int64_t value);
/*
 * Batches of independent instances (no reference counterpart: the reference
 * runs one tissue model per job).  The n contexts run concurrently, each
 * driven by its own host thread on its own stream, so the device overlaps
 * the instances' kernels.  Each context is used by one thread only; list a
 * context once.  seeds[i] seeds instance i.  tam_batch_step_coupled runs
 * `iters` outer iterations on every instance; tam_batch_run runs each
 * instance's whole loop as tam_run does (iters, nullable, receives the
 * per-instance iteration counts).  Both wait for every instance and check
 * each one's device error word; on failure the first failing instance's status
 * is returned and tam_last_error(NULL) names it (its own context holds the
 * message too).
 */
int tam_batch_step_coupled(struct tam_ctx *const *ctxs, int32_t n, int32_t iters, const uint64_t *seeds);
/* nsteps heat steps of every instance in persistent launches that each
 * advance all instances by a chunk of steps (FP32 config-mode contexts on one
 * device whose thermal properties are those of their material classes;
 * TAM_E_STATE otherwise).  tam_batch_step_coupled and tam_batch_run use the
 * same batched heat step whenever every context qualifies; MC passes and
 * re-trace decisions then happen at chunk boundaries. */
int tam_batch_heat_steps(struct tam_ctx *const *ctxs, int32_t n, int32_t nsteps);
/* One MC pass of every instance (tam_mc_pass of each, without the output
 * copy): nphotons[i] packets (nphotons NULL: each context's nphotons x
 * numproc), Philox key seeds[i] and stream streams[i] (streams NULL: each
 * context's count of passes so far, as the coupled loop uses).  The passes of
 * FP32 config-mode instances in a uniform medium on ctxs[0]'s device, with
 * the FP64 tally, run together in launches of a batched transport kernel (up
 * to 64 instances each; "batch.transport" 0 on ctxs[0] turns this off): its
 * packets draw from each instance's own Philox stream, so every instance's
 * tallies equal those of its own pass up to the order of the atomic sums.
 * The other instances' passes run one by one.  Waits for every instance and
 * checks its device error word.  tam_batch_step_coupled and tam_batch_run
 * run their passes the same way. */
int tam_batch_mc_pass(struct tam_ctx *const *ctxs, int32_t n, const int64_t *nphotons, const uint64_t *seeds,
                      const uint32_t *streams);
int tam_batch_run(struct tam_ctx *const *ctxs, int32_t n, const uint64_t *seeds, int64_t max_iters, int64_t *iters);

/*
 * Checkpoint / resume (no reference counterpart: the reference restarts from
 * input.params).  tam_save_state writes every device field of the context in
 * its storage precision together with the clock, pulse state and counters,
 * so a context created with the same parameters and configuration continues
 * bit for bit after tam_load_state (TAM_E_STATE if they differ).
 */
int tam_save_state(struct tam_ctx *ctx, const char *path);
int tam_load_state(struct tam_ctx *ctx, const char *path);

/*
 * Autotuner (no reference counterpart).  Config mode: times the context's own
 * workload under candidate settings of "transport.scat_min" (an MC pass of
 * `packets`) and of "heat.zchunk" / "heat.slab" / "heat.cls_rows" (`steps`
 * heat steps), keeps the fastest and puts the context's state back as it was
 * (fields, clock, pulse state, tallies).  0 packets or 0 steps skips that
 * part.  chosen (nullable) receives up to nchosen values: scat_min, zchunk,
 * cls_rows, slab.
 */
int tam_autotune(struct tam_ctx *ctx, int64_t packets, int32_t steps, int64_t *chosen, int32_t nchosen);
/* Autotuner of the batched heat step: times `steps` batched steps of the n
 * contexts (as tam_batch_heat_steps requires them) for each candidate form
 * and z-chunk length ("batch.staged" 4 with "batch.zchunk" 16..64, 3 with
 * 8..32, 2 or 1 with 8..64), keeps the
 * fastest on ctxs[0] (whose settings the batch reads) and puts every
 * instance's state back.  The candidates include the streams form
 * ("batch.streams" 1).  chosen (nullable): staged form, z-chunk, streams. */
int tam_batch_autotune(struct tam_ctx *const *ctxs, int32_t n, int32_t steps, int64_t *chosen, int32_t nchosen);

/* Kernels this library has launched in this process (all contexts). */
int64_t tam_kernel_launches(void);

/* writer (src/writer.f90:6-81): stream-unformatted FP64 files in `dir`. */
int tam_write_output(struct tam_ctx *ctx, const char *dir);

/*
 * Allocation-free MC pass.  No counterpart in the reference: the reference
 * allocates its module arrays itself and never runs on a GPU.  Some callers
 * cannot let this library call cudaMalloc -- a Fortran host whose device
 * arrays belong to another runtime (OpenACC, CUDA Fortran) that must not see
 * the device heap change behind its back, or a host working within a fixed
 * device-memory budget.  This entry point allocates nothing: the caller
 * passes the reference-mode parameters, `rhokap` as a device pointer in the
 * halo layout ((nx+2)(ny+2)(nz+2) doubles, input) and `jmean_global` as a
 * device pointer (nx*ny*nz doubles, output), plus the laser power `power` (W)
 * of the normalisation of src/mcpolar.f90:174.  It runs the same photon loop
 * as tam_mc_pass in reference mode (p->precision selects the FP64 or FP32
 * transport), on `cuda_stream` (NULL: the legacy default stream), and is
 * synchronous: it reads the pass's error word back and returns after that
 * stream has finished the pass.
 * The device is the caller's current device, and p->device must name it
 * (otherwise TAM_E_INVALID); the library does not change the current device.
 * The pass's scratch lives in one file-scope device array sized for grids of
 * at most TAM_NOALLOC_MAX_VOXELS voxels (about 16 MiB, held by every GPU that
 * loads the library until the process exits); larger grids are rejected with
 * TAM_E_INVALID.  The first call on a device looks up the array's device
 * address and keeps it for the rest of the process, so make that first call
 * before any stream capture, and do not reset that device (cudaDeviceReset)
 * afterwards.  All calls share the array (it is cleared at the start of each
 * call): calls that overlap on the GPU race.  Errors are reported by
 * tam_last_error(NULL).
 */
#define TAM_NOALLOC_MAX_VOXELS 2097152
int tam_mc_pass_noalloc(const tam_params *p, const double *rhokap, double *jmean_global, int64_t nphotons,
                        uint64_t seed, uint32_t stream, double power, void *cuda_stream);

/* Measurement (no reference counterpart): the current device's rate of
 * fire-and-forget atomic adds (FP64, or FP32 with fp32 != 0) into a tally of
 * `cells` entries at cells drawn from Philox inside the kernel, launched as
 * the transport kernel is (4 blocks of 256 threads per SM): the ceiling of
 * the transport's tally updates.  Allocates and frees its own tally. */
int tam_measure_tally_atomics(int64_t cells, int32_t fp32, double *per_second);

/* Self-test: Philox4x32-10 of this library against cuRAND's device Philox on
 * n inputs of 6 words {c0,c1,c2,c3,k0,k1}; outputs 4 words each. */
int tam_selftest_philox(const uint32_t *in, uint32_t *out_mine, uint32_t *out_curand, int64_t n);

#ifdef __cplusplus
}
#endif
#endif /* TAM_H */
