// tam_kernels.h -- argument blocks and launchers of the sm_103a kernels.
// Host-only declarations (no device code), included by the C-ABI layer.
#pragma once

#include <cstdint>
#include <string>

#include <cuda_runtime.h>

namespace tam {

// Kernel launches issued by this library (process-wide).
void count_launch(int n = 1);
int64_t launch_count();
// Message returned by tam_last_error(NULL) on this thread.
void set_thread_error(const std::string &msg);

constexpr int MAX_MAT = 16;
constexpr int FX_TILE = 32, FY_TILE = 8;  // x / y tile (thread block) of the fused heat kernels

enum Medium : int32_t { MED_RHOKAP = 0, MED_MATERIAL = 1, MED_UNIFORM = 2 };
enum Source : int32_t { SRC_DISK = 0, SRC_GAUSSIAN = 1 };

// Tally slots (double), same order as the oracle's ORC_T_*.
enum Tally : int {
    T_ABSORBED = 0, T_SPECULAR, T_REFLECTED, T_TRANSMITTED, T_SIDE, T_ROULETTE_NET, T_MISSED,
    T_STEPS, T_SCATTERS, T_OVERFLOW, N_TALLY
};

struct OptMat {
    double mua, mus, g, n;
};

// Values of one reference-mode outer iteration that change from iteration to
// iteration, read by the kernels from device memory when an iteration is
// replayed from a CUDA graph (the pointers below are then set).
struct RefIterVals {
    double f;          // normalisation of the iteration's MC pass, (P/81)/(N V)
    double laser_on;   // laserOn of its heat step
    double time;       // clock after its heat step (threshold time stamps)
    uint32_t stream;   // Philox stream of its MC pass (the iteration counter)
};

// One transport pass (packets [p0, p0 + n)).
// Per-launch constants of the transport kernel in the working precision,
// computed once on the host by launch_transport (its IEEE double operations
// give the bits a thread would compute), so no thread spends FP64 divisions
// on them.
template <typename Real> struct TrConst {
    Real hx, hy, hz;                  // cell widths 2 max / n
    Real knx, kny, knz;               // 1 - nudge / h: a crossed axis's next face after the nudge
    Real w2x, w2y;                    // 2 xmax, 2 ymax
    Real xmax, ymax;
    Real wmin, rm, inv_rm;            // roulette threshold, survival factor and its inverse
    Real namb, rhokap_n, src_r;       // ambient and rhokap-medium refractive indices, source radius
};

struct TransportArgs {
    int32_t nx, ny, nz;
    double xmax, ymax, zmax;          // half-widths, cm
    int32_t medium;                   // Medium
    const double *rhokap;             // halo (nx+2)(ny+2)(nz+2), MED_RHOKAP
    const uint8_t *mat;               // interior nx*ny*nz, MED_MATERIAL
    const uint8_t *btab;              // MED_MATERIAL, nullable: per 8^3 brick its one material id, or 0xFF
    int32_t bbx, bby;                 // bricks along x and y
    int32_t nmat;
    OptMat lut[MAX_MAT];
    double rhokap_n;                  // refractive index of the rhokap medium
    double n_ambient;
    int32_t source;                   // Source
    double source_radius;             // cm
    int32_t fresnel, roulette;
    double roulette_w, roulette_m;
    uint64_t seed;
    uint32_t stream;
    const uint32_t *stream_dev;       // non-null: the stream is read from here
    int64_t p0, n;
    int64_t max_steps;
    double nudge;                     // offset past a crossed face (reference delta), 0 in config mode
    int32_t scat_min;                 // lanes that must wait before a warp scatters (0: default)
    int32_t uniform_id;               // >= 0: every voxel holds this material (no per-cell fetch)
    double *jmean;                    // interior, packet units (sum of w*d*mua)
    float *jmean32;                   // non-null: deposits inside the box below go here in FP32 (the host
                                      // flushes them into jmean); deposits outside it go to jmean in FP64
    int32_t bx0, by0, bz0;            // the FP32 tally's box: first cell and extent per axis
    int32_t bnx, bny, bnz;
    double *tally;                    // N_TALLY doubles
    unsigned long long *work;         // dynamic packet counter (zeroed by the launcher)
    unsigned *err;                    // device error word
    TrConst<double> cd;               // filled by launch_transport
    TrConst<float> cf;
    uint32_t rk[20];                  // Philox round keys of `seed`, filled by launch_transport
};

// One instance of a batched FP32 transport pass (config mode, a uniform
// medium, the FP64 tally): its grid, beam and material, its Philox key and
// stream, and its packets' place in the batch's concatenated packet range.
struct BatchTrInst {
    int32_t nx, ny, nz;
    int32_t source, fresnel, roulette;
    float hx, hy, hz, w2x, w2y, xmax, ymax, src_r, namb;
    float wmin, rm, inv_rm;
    float mut, mua, alb, g, g2, n;    // the instance's material
    float inv_mut;                    // 1 / mut (a flight's distance is its optical depth times this)
    uint64_t seed;
    uint32_t stream, max_steps;
    int64_t first, count;             // its packets are [first, first + count) of the batch
    double *jmean;                    // interior, packet units
    double *tally;                    // N_TALLY doubles
    unsigned *err;                    // the instance's device error word
};
constexpr int MAX_BATCH_TR = 64;      // instances per batched launch
// An instance's entry from the arguments of its own FP32 uniform-medium pass
// (the batch's `first` is left 0 for the caller to set).
void fill_batch_inst(const TransportArgs &a, BatchTrInst &b);
// One launch for up to MAX_BATCH_TR instances (insts: a device copy of the
// table): every packet sees the streams and the arithmetic of its instance's
// own single pass (transport_kernel<float, uniform>), so the tallies agree up
// to the order of their atomic sums.
cudaError_t launch_batch_transport(const BatchTrInst *insts, int n, int64_t total, unsigned long long *work,
                                   int scat_min, int sm_count, cudaStream_t s);

// Launch the transport kernel in FP32 (fp64 == false) or FP64.
cudaError_t launch_transport(const TransportArgs &a, bool fp64, int sm_count, cudaStream_t s);
// Brick table of a material grid for the transport's cell lookups: for every
// 8 x 8 x 8 brick (bricks ceil(n / 8) per axis, x fastest) the material id all
// its voxels inside the grid hold, or 0xFF.
int64_t brick_table_size(int nx, int ny, int nz);
cudaError_t launch_brick_table(const uint8_t *mat, int nx, int ny, int nz, uint8_t *btab, cudaStream_t s);

// acc[cell of q] += (double)part[q], part[q] = 0 for the bnx x bny x bnz box
// of cells starting at (bx0, by0, bz0) in an nx x ny grid (flush of the
// FP32 box tally; part is box-indexed, x fastest).
cudaError_t launch_flush_f32(double *acc, float *part, int nx, int ny, int bx0, int by0, int bz0, int bnx, int bny,
                             int bnz, cudaStream_t s);

// out[q] = in[q] * f for q < n; in is then zeroed when zero_in is set.
// out = in * f; with `sum`, also *sum += the total of in (the caller zeroes *sum)
cudaError_t launch_scale_f64(double *out, double *in, double f, int64_t n, bool zero_in, cudaStream_t s,
                             double *sum = nullptr, const double *f_dev = nullptr);
cudaError_t launch_scale_to_f32(float *out, double *in, double f, int64_t n, bool zero_in, cudaStream_t s,
                                double *sum = nullptr);

// Atomic-add ceiling of the tally: blocks x 256 threads, per_thread (a
// multiple of 4) adds of 1 each at Philox-drawn cells of acc[0, cells).
cudaError_t launch_atomic_peak(void *acc, bool fp32, uint32_t cells, int blocks, int per_thread, uint32_t seed,
                               cudaStream_t s);

// Philox self-test: out_mine / out_curand hold 4 words per input; in holds 6
// words per input {c0, c1, c2, c3, k0, k1}.
cudaError_t launch_philox_selftest(const uint32_t *in, uint32_t *out_mine, uint32_t *out_curand, int64_t n,
                                   cudaStream_t s);

// ---------------------------------------------- reference-mode heat path --
// Scalars of module Heat (src/3dFD.f90:7-12) needed on the device.
struct RefHeatArgs {
    int32_t nx, ny, nz;
    double idx2, idy2, idz2;          // 1/dx^2 etc (dx = 2 max 1e-2 / (n+2))
    double delt, laserOn, vvox, mvox, qvapor;
    const double *t0;                 // halo, read
    double *tn;                       // halo, written (interior)
    const double *kappa, *density, *heatcap, *coeff; // halo
    const double *J;                  // interior jmeanGLOBAL
    double *Q;                        // interior
    unsigned *err;
    int32_t f32;                      // 1: the FP32 form, on the FP32 copies below
    int64_t nh;                       // halo cells per field
    const float *p32;                 // FP32 kappa, density, heatcap, coeff (4 x nh)
    const float *s0;                  // FP32 copy of t0
    float *sn;                        // FP32 copy of tn, written with it
    const double *laser_dev;          // non-null: laserOn is read from here
};
cudaError_t launch_ref_stencil(const RefHeatArgs &a, cudaStream_t s);

struct RefArrheniusArgs {
    int32_t nx, ny, nz;
    double delt, time;
    const double *time_dev;           // non-null: the time stamp is read from here
    const double *temp, *rhokap;      // halo
    double *tissue, *thres;           // interior, interior x 3
};
cudaError_t launch_ref_arrhenius(const RefArrheniusArgs &a, cudaStream_t s);

struct RefPropsArgs {
    int32_t nx, ny, nz;
    double abl_T, delt, qvapor, mu_water, mu_protein;  // abl_T: ablation temperature + 273 (kelvin)
    const double *temp;               // halo
    const double *rk_old;             // halo
    double *rk_new;                   // halo (interior written)
    double *kappa, *density, *heatcap, *coeff, *alpha; // halo
    const double *Q;                  // interior
    double *water;                    // interior
    unsigned *err;
    int32_t reuse;                    // 1: the previous call's skin properties are intact (same delt)
    float *p32;                       // null, or FP32 copies of kappa, density, heatcap, coeff (4 x nh)
    int64_t nh;
};
cudaError_t launch_ref_props(const RefPropsArgs &a, cudaStream_t s);
// Arrhenius and then the property update of every voxel in one pass (their
// outputs are disjoint and the update reads no damage)
cudaError_t launch_ref_damage_props(const RefArrheniusArgs &d, const RefPropsArgs &a, cudaStream_t s);

// FP32 copies for the FP32 form of the reference stencil: T into both
// t32a and t32b (halo included), kappa, density, heatcap, coeff into p32
cudaError_t launch_ref_shadow(int64_t nh, const double *T, float *t32a, float *t32b, const double *kappa,
                              const double *density, const double *heatcap, const double *coeff, float *p32,
                              cudaStream_t s);

// tissue(rhokap <= 0.1) = -1 (src/mcpolar.f90:196-204)
cudaError_t launch_ref_finalize(int nx, int ny, int nz, const double *rhokap, double *tissue, cudaStream_t s);

// --------------------------------------------------- fused config-mode step --
enum Bc : int32_t { BC_DIRICHLET = 0, BC_ROBIN = 1 };

// Slots of the pre-converted constant table of the fused step.
enum FusedConst : int {
    FC_CX = 0, FC_CY, FC_CZ,          // opscale / d^2 per axis
    FC_DT, FC_PDT, FC_VVOX, FC_TBOIL, FC_LW, FC_TLO_S, FC_TABL_S, FC_SCREEN,
    FC_BCT = 11,                      // 6 Dirichlet face temperatures
    FC_BCHD = 17,                     // 6 Robin h * d (d: spacing normal to the face)
    FC_BCTA = 23,                     // 6 Robin ambient temperatures
    // Arrhenius constants for the FP32 form: ln A and Ea/R as float-float
    // pairs (high part, low part), exact window and ablation temperatures
    FC_LNA_HI = 29, FC_LNA_LO, FC_EAR_HI, FC_EAR_LO, FC_TLO, FC_THI, FC_TABL,
    FC_TLO_LO, FC_THI_LO, FC_TABL_LO, // low parts of the three temperatures
    // FP32 Kahan term of the clamped boiling temperature: the pair
    // (FC_TBOIL, FC_TBOIL_E) has the true value T_boil (true T = T - e)
    FC_TBOIL_E = 39,
    FC_N = 40
};

// Values of one heat step that change from step to step, read by the fused
// kernels from device memory when FusedArgs::sv is set (graph-captured steps).
struct StepVals {
    double pdt;                       // source multiplier x dt of the step
    double t_new;                     // time stamp at the end of the step
};

struct FusedArgs {
    int32_t nx, ny, nz;
    double dx, dy, dz;                // m
    double opscale, dt, vvox;
    int32_t boil;
    double T_boil, lw, T_abl;
    int32_t arrhenius;
    double lnA, Ea, Rgas, T_lo, T_hi, thr[3];
    int32_t bc_type[6];
    double bc_T[6], bc_h[6], bc_Tamb[6];
    double P;                         // source multiplier for this step
    double t_new;                     // time stamp of this step's end
    const StepVals *sv;               // non-null: P dt and t_new of this step come from here
    const void *T_in;                 // interior, Real
    void *T_out;
    const float *Tc_in;               // Kahan compensation (FP32 form only)
    float *Tc_out;
    const void *k, *rho, *c;          // Real
    void *J, *Q;                      // Real
    double *omega, *thres;
    uint8_t *mat;
    unsigned long long *n_ablated;    // running count
    unsigned *err;
    int32_t zchunk;                   // z planes per thread column (0: automatic)
    int32_t arr_fp64;                 // FP32 form: 1 = Arrhenius exponent in FP64, 0 = float-float
    // the constants above in the kernel's storage precision (filled by
    // launch_fused_step), so the kernel converts nothing per voxel
    float fc[FC_N];
    double dc[FC_N];
};
// fp64 == false: FP32 storage with Kahan compensation; true: plain FP64.
cudaError_t launch_fused_step(const FusedArgs &a, bool fp64, cudaStream_t s);
// Fill FusedArgs::fc / dc from the physical constants.
void fill_fused_consts(FusedArgs &a);

// TMA form of the FP32 fused step.  Needs nx * 4 bytes to be a multiple of
// 16 (TMA row strides); tensor maps are built once per buffer set.
struct FusedTma;  // opaque: tensor maps of T[2], Tc[2], Ax, Ay, Az, 1/(rho c), J
bool fused_tma_supported(int nx);
cudaError_t fused_tma_create(FusedTma **out, int nx, int ny, int nz, float *const T[2], float *const Tc[2],
                             const float *ax, const float *ay, const float *az, const float *irc, const float *J);
// Face coefficients (and 1/(rho c)) of the TMA form from k, rho, c.
cudaError_t launch_face_coeffs(const FusedArgs &a, float *ax, float *ay, float *az, float *irc, cudaStream_t s);
void fused_tma_destroy(FusedTma *m);
// `which` selects the (T, Tc) buffer pair read by this step (0 or 1).
cudaError_t launch_fused_tma(const FusedArgs &a, const FusedTma *m, int which, cudaStream_t s);

// Class-table form of the FP32 TMA step: thermal properties given per class
// (material) and a u8 class id per voxel, stored with a row pitch that is a
// multiple of 16 bytes (cls_pitch_for).  No coefficient arrays are read.
struct ClassLut {
    float fa[MAX_MAT * MAX_MAT];  // k_f / (rho_f c_f) of the face between classes i and j (arithmetic means)
    float irc[MAX_MAT];           // 1 / (rho c)
    float k[MAX_MAT], rho[MAX_MAT], c[MAX_MAT];
    int32_t uniform;              // >= 0: every voxel has this class
};
struct FusedCls;  // opaque: tensor maps of T[2], Tc[2], J and the class grid
int cls_pitch_for(int nx);
cudaError_t launch_cls_from_mat(const uint8_t *mat, int nmat, uint8_t *cls, int nx, int ny, int nz, int pitch,
                                cudaStream_t s);
cudaError_t fused_cls_create(FusedCls **out, int nx, int ny, int nz, float *const T[2], float *const Tc[2],
                             const float *J, const uint8_t *cls, int pitch);
void fused_cls_destroy(FusedCls *m);
// rows: voxel rows per thread (1 or 2).
cudaError_t launch_fused_cls(const FusedArgs &a, const FusedCls *m, int which, const ClassLut &L, int rows,
                             cudaStream_t s);

// Slab form of the FP32 class-table step (heat_slab.cu): tiles of 32 x 8
// voxels, voxel pairs, one block barrier per plane, boundary faces as ghost
// neighbours in the staged planes, rare voxels (boiling, damage window,
// ablation) redone from a per-block list after the planes.  Same layout
// requirements as the class-table form (nx a multiple of 4, class rows of a
// 16-byte pitch) and fewer than 2^31 voxels.
struct FusedSlab;  // opaque: tensor maps of T[2], Tc[2], J and the class grid
bool fused_slab_supported(int nx, int ny, int nz);
cudaError_t fused_slab_create(FusedSlab **out, int nx, int ny, int nz, float *const T[2], float *const Tc[2],
                              const float *J, const uint8_t *cls, int pitch);
void fused_slab_destroy(FusedSlab *m);
// Heterogeneous grids: recompute the slab form's per-(tile, plane) one-class
// flags from the class grid given at creation and, for the launch at
// `zchunk`, the lists of blocks whose tile, rim and planes hold one class
// (run by the one-class kernel with that class) and of the others (the class
// kernel).  Call after every change of the class grid or of the z-chunk;
// synchronises the stream.  Without lists for the launch's z-chunk the class
// kernel takes every block.  fused_slab_generation counts the rebuilds.
cudaError_t fused_slab_tile_flags(FusedSlab *m, int zchunk, cudaStream_t s);
unsigned fused_slab_generation(const FusedSlab *m);
cudaError_t launch_fused_slab(const FusedArgs &a, const FusedSlab *m, int which, const ClassLut &L, cudaStream_t s);

// Batched FP32 heat step of many instances in one persistent cooperative
// launch (batch.cu).  BatchInst lives in device memory, one per instance.
struct BatchInst {
    FusedArgs a;                  // constants filled by fill_fused_consts; the instance's buffers
    ClassLut L;
    const uint8_t *cls;           // class grid, rows of cls_pitch bytes
    int32_t cls_pitch;
    float *T[2], *E[2];           // temperature and Kahan-term buffer pairs
    int32_t fcur;                 // pair read by the first step of the launch
    int32_t tiles_x, tiles_y, zchunk;
};
struct BatchStep {                // per step and instance
    double t_new;                 // time stamp at the end of the step
    float pdt;                    // laser power * dt of the step (0: source off)
    int32_t active;               // 0: the instance does not step
};
struct BatchSync {
    unsigned count, gen, abort;
};
// Resident blocks of the batched kernel on the current device (its grid size);
// staged: 2 = planes staged in shared memory by cp.async, a pair of voxels
// per thread; 1 = the same with one voxel per thread; 0 = neighbours read
// with cached global loads.
cudaError_t batch_heat_blocks(int *blocks, int staged);
// K steps of every instance; prefix[i] = first work item of instance i,
// prefix[n] = total work items; steps is K x n (step-major).
cudaError_t launch_batch_heat(const BatchInst *insts, int n, const int *prefix, const BatchStep *steps, int K,
                              BatchSync *sync, unsigned *err, int blocks, int staged, cudaStream_t s);
// The slab form of the batched step (batch.staged 3): z-chunks of at most
// BATCH_SLAB_ZMAX planes (BatchInst::zchunk), rows of any pitch staged by
// 16-byte copies of the aligned chunks that cover them (the arrays need 256
// bytes of slack at both ends), voxels needing rare work handled after each
// item.  uniform: every instance's grid is one material class.
constexpr int BATCH_SLAB_ZMAX = 32;
cudaError_t batch_slab_blocks(int *blocks, bool uniform);
cudaError_t launch_batch_slab(const BatchInst *insts, int n, const int *prefix, const BatchStep *steps, int K,
                              BatchSync *sync, unsigned *err, int blocks, bool uniform, cudaStream_t s);
// The same step with one launch per step (batch.staged 4): a block per work
// item (items = prefix[n]; zmax: the longest item's planes, at most
// BATCH_STEP_ZMAX), then a kernel over the step's list of rare voxels (rare:
// room for every voxel of the batch, as indices from vox0[i], the first voxel
// of instance i; rare_cnt: the list's length, zeroed before each step).
constexpr int BATCH_STEP_ZMAX = 128;
cudaError_t launch_batch_slab_steps(const BatchInst *insts, int n, const int *prefix, int items, int zmax,
                                    const int *vox0, const BatchStep *steps, int K, unsigned *rare,
                                    unsigned *rare_cnt, unsigned *err, bool uniform, int sm_count, cudaStream_t s);
// One step of one instance (inst: device copy of its BatchInst) by the staged
// voxel-pair kernel, one block per work item (prefix = {0, items}); any row
// pitch.  fcur selects the buffer pair read by the step.
cudaError_t launch_staged_step(const BatchInst *inst, const int *prefix, int items, const BatchStep &step, int fcur,
                               cudaStream_t s);

// The isolation rule of src/3dFD.f90:347-349 on the config-mode material
// grid: a voxel that is not air (id != 0) and whose six neighbours are air
// (outside the grid counts as air) becomes air, its source J (Real: double
// when fp64, else float) goes to zero and n_ablated counts it.  Updating in
// place equals the reference's sequential sweep: a voxel that turns to air
// here has only air around it, so no other voxel's test depends on it.
cudaError_t launch_isolate(uint8_t *mat, void *J, bool fp64, int nx, int ny, int nz, unsigned long long *n_ablated,
                           cudaStream_t s);

// Halo (reference-layout) FP64 temperature from the interior state, with
// ghosts filled from the boundary conditions.
cudaError_t launch_fused_to_halo(const FusedArgs &a, bool fp64, double *halo, cudaStream_t s);
// Interior Real state from a halo FP64 temperature (Tc zeroed).
cudaError_t launch_fused_from_halo(const FusedArgs &a, bool fp64, const double *halo, cudaStream_t s);

}  // namespace tam
