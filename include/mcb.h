/*
 * mcb.h - C ABI of the GB300-native phase-field lattice-Boltzmann bubble solver.
 *
 * The library advances two D3Q19 lattices per update, as the reference's step loop does
 * (src/main.cu:74-190 of kreeyto/MULTIC-BUBBLE-CUDA):
 *   - g carries a conservative Allen-Cahn phase field phi;
 *   - f carries the flow, with regularized collision and He-style surface-tension forcing.
 * The ten launches of that loop (src/lbm.cu:5-461) become one fused sm_103a kernel per
 * update. It computes normals, curvature, force, moments, the regularized f collision and
 * the g collision, pull-streams f, and adds each cell's exact integer g populations into
 * the next update's phi (the pull-stream of g and the phi sum of the reference). Only the
 * opt-in TMA variant, and the first update with stored g, run a separate phi kernel.
 *
 * Conventions:
 *   - Every call returns an int status: MCB_OK (0) or one of MCB_ERR_*. The reference
 *     ignores every CUDA return code. mcb_last_error() gives the message of the last
 *     failure on the calling thread.
 *   - Fields are float32, nx*ny*nz cells, x fastest: index i + nx*(j + ny*k). This is the
 *     reference's inline3D (src/header.cuh:22-24) and dump order (src/auxFunctions.cu:49-67).
 *   - A handle owns all of its device memory (the reference keeps 22 process-global
 *     arrays, src/var.cu:57-114). Calls on one handle must come from one host thread at a
 *     time. They are ordered on the handle's own CUDA stream.
 *   - "Update s" follows the reference's numbering: phi, rho and u of update s are the
 *     values computed at the start of update s. After mcb_step(h, n) on a fresh handle,
 *     the fields are those of update n-1. That is what the reference dumps at STEP = n-1.
 */
#ifndef MCB_H
#define MCB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MCB_ABI_VERSION 4

/* status codes */
#define MCB_OK            0
#define MCB_ERR_INVALID   1  /* bad argument or configuration */
#define MCB_ERR_CUDA      2  /* a CUDA runtime call failed */
#define MCB_ERR_ALLOC     3  /* device or host allocation failed */
#define MCB_ERR_IO        4  /* file could not be written */
#define MCB_ERR_STATE     5  /* call out of order (e.g. step before fields are set) */
#define MCB_ERR_NUMERIC   6  /* NaN or Inf found by the diagnostics */

/* boundary handling */
#define MCB_BC_REF        0  /* the reference's frozen 1-cell shell: rest-equilibrium inflow
                                (src/lbm.cu:365-401), zero-gradient shell phi lagged by one
                                update (src/lbm.cu:403-425), shell cells never collide.
                                Requires g relaxation tau_g = 1 as in src/lbm.cu:290-329. */
#define MCB_BC_PERIODIC   1  /* periodic in x, y and z */
#define MCB_BC_WALLS_Z    2  /* periodic in x and y, half-way bounce-back walls at z = -1/2
                                and z = nz-1/2 (no-slip for f, no-flux for g) */

/* population storage (arithmetic is FP32 in every case) */
#define MCB_STORE_F32     0  /* f: float32; g: 32-bit fixed point Q2.30 (exact phi mass) */
#define MCB_STORE_F16     1  /* f, g: float16 deviation form; g rest population Q2.30 */
#define MCB_STORE_BF16    2  /* f, g: bfloat16 deviation form; g rest population Q2.30 */

/* fields for mcb_get_field */
#define MCB_FIELD_PHI     0
#define MCB_FIELD_RHO     1
#define MCB_FIELD_UX      2
#define MCB_FIELD_UY      3
#define MCB_FIELD_UZ      4
#define MCB_FIELD_P       5  /* p = rho * cs^2, cs^2 = 1/3 */

/* One simulation case. The reference hard-codes these values in src/var.cu:3-25,
 * src/init.cu:39,46 and src/main.cu:35. */
typedef struct mcb_config {
    int   nx, ny, nz;   /* lattice size; each >= 4 (>= 8 for MCB_BC_REF) */
    int   bc;           /* MCB_BC_* */
    int   storage;      /* MCB_STORE_* */
    float tau;          /* f relaxation time; omega = 1/tau (src/var.cu:21-23) */
    float tau_g;        /* g relaxation time; 1 = full relaxation (src/lbm.cu:290-329) */
    float sigma;        /* surface tension (src/var.cu:25) */
    float width;        /* interface width W of the tanh profile */
    float sharp_c;      /* g sharpening coefficient; <= 0 means (tau_g - 1/2) * 4 / width.
                           The reference's value is 0.45 (src/var.cu:24). */
    float gravity;      /* Boussinesq buoyancy: F_z += gravity * (phi - mean phi); 0 = off */
    int   device;       /* CUDA device ordinal */
    int   variant;      /* kernel tile variant, -1 = default (see mcb_variant_count) */
    int   zchunk;       /* work split: > 0 fixed chunks of zchunk z planes per block;
                           -w (w <= 16) balanced over w waves of resident blocks, each
                           block taking an equal run of planes; 0 = default (one wave of
                           equal chunks when one case's tile columns fit in it, else
                           32-plane chunks) */
    int   use_graph;    /* 1 = replay updates from a CUDA graph, 0 = plain launches */
    int   g_mode;       /* how g crosses between updates:
                           MCB_G_AUTO: with tau_g = 1 every post-collision g population is
                             the equilibrium W_l (phi + c_l.J) of its cell,
                             J = 3 phi u + sharp_c phi (1 - phi) n: the collide kernel adds
                             the 19 populations, as exact Q2.30 integers, straight into the
                             next update's phi and no g is stored (the TMA variant stores
                             (phi, J) per cell and rebuilds them); with tau_g != 1 all 19
                             are stored;
                           MCB_G_POPULATIONS: always store the 19 populations. */
    int   velocity_set; /* velocity set of f: 19 (D3Q19, the reference's build) or 27
                           (D3Q27 with the tables of src/var.cu:33-35,47-52; the
                           reference's D3Q27 moments are unfinished, src/lbm.cu:174-218).
                           g and the phi stencils are D3Q19 either way. D3Q27 runs the
                           32x8 tile. */
    float rho_in;       /* density of the phi = 1 phase (the bubble) */
    float rho_out;      /* density of the phi = 0 phase. rho_in == rho_out (default 1, 1)
                           runs the reference's density-matched update; otherwise f carries
                           the normalised pressure p / (rho cs^2) of the velocity-based
                           density-ratio formulation (Zu and He 2013; Fakhari et al. 2017),
                           with rho = rho_out + (rho_in - rho_out) phi, one kinematic
                           viscosity, and MCB_FIELD_RHO reporting p / cs^2. Periodic and
                           wall modes only; runs the 32x8 tile. */
} mcb_config;

#define MCB_G_AUTO         0
#define MCB_G_POPULATIONS  1

/* FP64 diagnostics, reduced on the device in a fixed order (deterministic). */
typedef struct mcb_diag {
    double  mass;         /* sum of phi over the lattice (interior only for MCB_BC_REF) */
    int64_t mass_q30;     /* the same sum as an exact Q2.30 integer */
    double  kinetic;      /* sum of 0.5 * rho * |u|^2 */
    double  umax;         /* max |u| */
    double  rho_in;       /* mean rho over cells with phi > 0.99 */
    double  rho_out;      /* mean rho over cells with phi < 0.01 */
    double  dp;           /* cs^2 * (rho_in - rho_out), the Laplace pressure jump */
    double  n_in, n_out;  /* cell counts of the two averages */
    double  vol_half;     /* number of cells with phi > 0.5 */
    double  phi_min, phi_max;
    int     finite;       /* 1 if every phi, rho and u was finite */
    int     update;       /* index of the update these values belong to */
} mcb_diag;

typedef struct mcb_handle mcb_handle;
typedef struct mcb_batch  mcb_batch;

/* Error text of the last failed call on this thread ("" if none). */
const char* mcb_last_error(void);
int  mcb_abi_version(void);

/* Fills cfg with the reference's constants: 64x64x256 (src/var.cu:3-4), tau 0.505,
 * sigma 0.1, sharp_c 0.45 (src/var.cu:21-25), tau_g 1, width 3 (src/init.cu:46),
 * MCB_BC_REF, MCB_STORE_F32. */
int  mcb_config_default(mcb_config* cfg);

/* Replaces initializeVars (src/var.cu:57-114): validates cfg, allocates every device
 * buffer of one case and creates the handle's stream. */
int  mcb_create(const mcb_config* cfg, mcb_handle** out);
int  mcb_destroy(mcb_handle* h);

/* Replaces initTensor/initPhase/initDist (src/init.cu:3-80). phi, ux, uy, uz are host
 * arrays of nx*ny*nz floats; ux/uy/uz may all be NULL (fluid at rest). rho starts at 1,
 * f at the second-order equilibrium of (rho, u), g at W_l*phi*(1 + 3 c_l.u). With
 * u = 0 these are the reference's f = W*rho and g = W*phi. Resets the update counter. */
int  mcb_set_fields(mcb_handle* h, const float* phi, const float* ux, const float* uy,
                    const float* uz);

/* Replaces one pass of the step loop body (src/main.cu:77-182), nsteps times.
 * Asynchronous on the handle's stream; the next mcb_get_field/mcb_diagnostics waits. */
int  mcb_step(mcb_handle* h, int nsteps);
int  mcb_synchronize(mcb_handle* h);

/* Copies one field of the latest update to a host array of nx*ny*nz floats. For
 * MCB_BC_REF the shell of phi holds the zero-gradient copy, as in the reference's dumps. */
int  mcb_get_field(mcb_handle* h, int which, float* host);

/* Copies the exact Q2.30 phi of the latest update (1.0 = 2^30) to a host array of nx*ny*nz
 * int32, x fastest. These are the integers whose sum (over the interior for MCB_BC_REF) is
 * mcb_diag.mass_q30. No counterpart in the reference, which keeps phi in float32. */
int  mcb_get_phi_q30(mcb_handle* h, int32_t* host);

/* FP64 reductions over the latest update (replaces the placeholders of
 * src/auxFunctions.cu:24-40). Returns MCB_ERR_NUMERIC, with out filled, if a value is
 * not finite. */
int  mcb_diagnostics(mcb_handle* h, mcb_diag* out);

/* Replaces copyAndSaveToBinary (src/auxFunctions.cu:49-67): writes phi of the latest
 * update to "<dir><id>_phi%06d.bin" as raw little-endian float32, nx*ny*nz values,
 * x fastest. post/fileTreat.py reads the file back. dir must end in a path separator,
 * as SIM_DIR does in src/main.cu:20-21. */
int  mcb_dump_phi(mcb_handle* h, const char* dir, const char* id, int step);

/* The same dump for any field of mcb_get_field: "<dir><id>_<name>%06d.bin", with name
 * phi, rho, ux, uy, uz or pres (p = rho/3; "pres" because post/fileTreat.py matches
 * file names by substring, and "p" is a substring of "phi"). The reference dumps phi
 * only; post/fileTreat.py:8 reads the others once they are added to __macr_names__. */
int  mcb_dump_field(mcb_handle* h, const char* dir, const char* id, int which, int step);

/* Replaces generateSimulationInfoFile (src/auxFunctions.cu:12-47): writes
 * "<dir><id>_info.txt" in the layout post/fileTreat.py:37-124 parses, with
 * "Precision: float" (the dump format). Measured MLUPS is written when mlups > 0. */
int  mcb_write_info(const mcb_handle* h, const char* dir, const char* id,
                    const char* velocity_set, int save_every, int nsteps, double mlups);

/* The two writers behind mcb_dump_phi and mcb_write_info, for host data (no GPU needed).
 * mcb_write_phi_file writes n floats to "<dir><id>_<name>%06d.bin"
 * (copyAndSaveToBinary, src/auxFunctions.cu:49-67). mcb_write_info_file writes the
 * info file of generateSimulationInfoFile (src/auxFunctions.cu:12-47). */
int  mcb_write_phi_file(const char* dir, const char* id, const char* name, int step,
                        const float* data, size_t n);
int  mcb_write_info_file(const char* dir, const char* id, const char* velocity_set,
                         int nx, int ny, int nz, double tau, double umax, double fx,
                         double fy, double fz, int save_every, int nsteps, double mlups);

/* The tile variant and z chunk setting the handle runs (after defaults and autotuning).
 * variant 4 is the TMA-staged 32x8 collide on the padded f layout; variant 5 takes two
 * neighbouring cells in x per thread (64x4 cells per block; D3Q19 f at density ratio 1 and
 * an even nx; with stored g also periodic or wall boundaries and 18 * cells < 2^31;
 * elsewhere a request for it runs variant 0), and variant 6 is variant 5 with an L2
 * prefetch of the f rows of the plane after next. Defaults: variant 5 where it applies
 * and its 64-cell-wide tiles are at least 85 % as full in x as 32-wide ones, except with
 * stored g below 2^18 cells (variant 0) and relaxed g (tau_g != 1: variant 6 at 16-bit
 * storage, variant 0 at FP32). With stored g the f layout follows the variant chosen
 * at creation: the autotuner then tries variants 5 and 6, or the one-cell ones, only. */
int  mcb_get_schedule(const mcb_handle* h, int* variant, int* zchunk);

/* Checkpoint and restart. No counterpart in the reference, which saves only phi
 * (src/main.cu:184-189) and so cannot resume. mcb_checkpoint_save writes everything the
 * next update reads:
 *   - the f populations, and the g populations (or the (phi, J) records of the TMA
 *     variant) where g is stored;
 *   - every phi buffer (two with the TMA variant, three with equilibrium g, four with
 *     stored g);
 *   - the fields of the latest update;
 *   - the update counter, the buffer parity and the buoyancy reference;
 * together with the configuration. mcb_checkpoint_load restores them into a handle created
 * with the same size, boundary mode, storage, g mode and f layout (MCB_ERR_INVALID
 * otherwise; the layout differs between the pair variants and the others with stored g,
 * and for the TMA variant). The run then continues bit-identically. The file is raw
 * little-endian. */
int  mcb_checkpoint_save(mcb_handle* h, const char* path);
int  mcb_checkpoint_load(mcb_handle* h, const char* path);

/* Number of updates run since mcb_set_fields, and the size of one case. */
int  mcb_get_update(const mcb_handle* h, int* update);
int  mcb_get_dims(const mcb_handle* h, int* nx, int* ny, int* nz);

/* Device time in milliseconds of the last mcb_step call (CUDA events on the handle's
 * stream around its launches). */
int  mcb_last_step_ms(mcb_handle* h, float* ms);

/* Like mcb_step, but with plain launches and a CUDA event after every kernel, for
 * measurement. On return: total_ms is the device time from the first launch to the last;
 * phi_ms is the summed time from the end of one update to its collide launch (the phi
 * kernel where there is one, else the gap between launches); collide_ms is the summed
 * duration of the collide kernels. */
int  mcb_step_profiled(mcb_handle* h, int nsteps, float* total_ms, float* phi_ms,
                       float* collide_ms);

/* Kernel tile variants: count and shape (threads in x and y per block). */
int  mcb_variant_count(void);
int  mcb_variant_shape(int variant, int* bx, int* by);

/* Times every tile variant and work split (the mcb_config.zchunk values 0, -1..-4, 8, 16,
 * 32) on a copy of the handle's state for nsteps updates each. Keeps the fastest in the
 * handle and reports it (best_zchunk 0: the default split) and its MLUPS. The handle's
 * fields are restored afterwards. */
int  mcb_autotune(mcb_handle* h, int nsteps, int* best_variant, int* best_zchunk,
                  double* best_mlups);

/* Allocation-free diagnostics over fields the caller keeps on the device.
 * No counterpart in the reference. It exists for callers that cannot call cudaMalloc:
 *   - a host code that owns all device memory through its own pool, sized at start-up;
 *   - a loop that must not risk the device-wide synchronisation cudaFree can imply.
 * It computes the reductions of mcb_diagnostics from:
 *   - phi, rho, ux, uy, uz: device arrays of nx*ny*nz floats, x fastest;
 *   - phi_q30: the matching Q2.30 phi (mcb_get_phi_q30 gives a handle's), or NULL to take
 *     the integer mass from phi rounded to Q2.30.
 * kinetic is 0.5 * rho * |u|^2 with rho the given rho field. That is what mcb_diagnostics
 * computes for density-matched cases. With a density ratio (rho_in != rho_out) a handle's
 * rho field holds p / cs^2, and mcb_diagnostics takes the density rho_out + (rho_in -
 * rho_out) phi instead, so the two kinetic energies differ there; every other value agrees.
 * It enqueues the reduction on `stream` (NULL: the default stream) and waits for the
 * result. bc = MCB_BC_REF leaves the shell out, as mcb_diagnostics does.
 * It allocates nothing on the device or the host. Its scratch is one file-scope device
 * array of 305 records (about 29 KB), fixed whatever the lattice size, and every GPU that
 * loads the library holds it until exit.
 * Every call looks up that array's device address in the current context with
 * cudaGetSymbolAddress (not a stream operation), so a context reset between calls is
 * harmless. The first call on a device may load the library's kernels into its context:
 * make that first call before any stream capture on the device.
 * All calls share the array. Calls that overlap on the GPU (other host threads, other
 * streams) race and must be serialised by the caller. No scratch needs clearing: every
 * block overwrites its own record. Lattices above MCB_DIAG_DEVICE_MAX_CELLS cells are
 * rejected with MCB_ERR_INVALID. */
#define MCB_DIAG_DEVICE_MAX_CELLS 2147483647LL
int  mcb_diagnostics_device(const float* phi, const float* rho, const float* ux,
                            const float* uy, const float* uz, const int32_t* phi_q30,
                            int nx, int ny, int nz, int bc, void* stream, mcb_diag* out);

/* ---- initial fields (host side; one generator shared by the GPU path and the tests) ---- */

/* One bubble: centre, radius and ellipsoid semi-axis factors (1,1,1 = sphere). */
typedef struct mcb_bubble {
    double cx, cy, cz, r;
    double ax, ay, az;
} mcb_bubble;

/* The reference's initPhase (src/init.cu:27-49): one bubble of radius r at
 * (nx/2, ny/2, nz/2), phi = 0.5 + 0.5 tanh(2 (r - |x - c|) / width) in float32 on
 * interior cells, shell cells 0. */
int  mcb_fill_phi_reference(int nx, int ny, int nz, float r, float width, float* phi);

/* phi = max over bubbles of 0.5 + 0.5 tanh(2 (R - d) / width). d is the distance to
 * the centre after dividing each axis offset by the bubble's semi-axis factor. Offsets
 * take the nearest periodic image in the periodic directions of bc. With MCB_BC_REF the
 * shell cells are 0, as the reference's init leaves them (src/init.cu:37). */
int  mcb_fill_phi_bubbles(int nx, int ny, int nz, int bc, float width,
                          const mcb_bubble* bubbles, int nbubbles, float* phi);

/* Seeded workload generator for the benchmark scenarios:
 *   0 the reference-parity case: frozen shell, 64^3, the reference's node-centred bubble
 *     (R 12, width 4), tau 0.8, sigma 0.1;
 *   1 static bubble 64^3; 2 rising perturbed bubble 128x128x256;
 *   3 32 bubbles 256^3 with velocity noise; 4 one case of the batched set (case_index);
 *   5 512 bubbles 512^3; 6 a 64^3 rerun of scenario 3's setting with 4 bubbles.
 * "Centred" bubbles sit at the geometric centre of the nodes, (n-1)/2.
 * Scale s > 0 multiplies every length (domain, radii, centres) so a scenario can be run
 * smaller; s = 1 is the full size. Writes cfg, then phi/ux/uy/uz if they are non-NULL
 * (nx*ny*nz floats each; call once with NULL to learn the size from cfg). All randomness
 * comes from splitmix64(seed). */
int  mcb_workload(int scenario, int case_index, uint64_t seed, double scale,
                  mcb_config* cfg, float* phi, float* ux, float* uy, float* uz);

/* ---- batched cases: many independent cases of uneven size in one launch per update ---- */

/* All cases must share storage; each keeps its own size, bc, tau, sigma, ... */
int  mcb_batch_create(const mcb_config* cases, int ncases, mcb_batch** out);
int  mcb_batch_destroy(mcb_batch* b);
int  mcb_batch_set_fields(mcb_batch* b, int case_index, const float* phi, const float* ux,
                          const float* uy, const float* uz);
int  mcb_batch_step(mcb_batch* b, int nsteps);
int  mcb_batch_get_field(mcb_batch* b, int case_index, int which, float* host);
int  mcb_batch_diagnostics(mcb_batch* b, int case_index, mcb_diag* out);
int  mcb_batch_last_step_ms(mcb_batch* b, float* ms);
/* Total lattice cells over all cases (for MLUPS). */
int  mcb_batch_cells(const mcb_batch* b, int64_t* cells);

/* Per-size-class tile choice for a batch. The reference launches every kernel with one fixed
 * 8x8x8 block shape (src/main.cu:43-46); here a batch can pick, for each size class (the
 * cases of one nx, ny, nz), the tile variant and z chunk that run that class fastest.
 * On a copy of the batch's state, for nsteps updates per trial, it times:
 *   - the untuned schedule (every case in one launch, the batch's variant and split);
 *   - each size class alone with every tile variant that fits and the z chunks
 *     0 (default), 8, 16, 24, 32, 48, 64;
 *   - the chosen classes combined: one launch per chosen variant, each case with its
 *     class's chunk, and one launch of every case with the variant that covers the most
 *     cells.
 * It keeps the fastest measured combination (or the untuned schedule if none beats it),
 * reports both MLUPS, and restores the fields. Results do not depend on the work split;
 * the one-cell tile variants give identical fields, and the two-cells-per-thread variant
 * agrees with them to FP32 rounding. */
int  mcb_batch_autotune(mcb_batch* b, int nsteps, double* default_mlups, double* tuned_mlups);

/* The tile variant and z chunk setting that case case_index of a batch runs. */
int  mcb_batch_get_schedule(const mcb_batch* b, int case_index, int* variant, int* zchunk);

#ifdef __cplusplus
}
#endif
#endif /* MCB_H */
