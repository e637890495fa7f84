/*
 * dropfluid.h — C ABI of the GB300-native staggered-MAC fluid step of the
 * drop-of-blood simulator (semi-Lagrangian advection, Casson viscosity,
 * divergence, geometric-multigrid pressure solve, projection, Lagrangian
 * parcel advection/splat and dye transport).
 *
 * The reference drives this path from its TypeScript engine class
 * (src/engine/BloodDropEngine.ts).  Each entry point below names the
 * reference interface it replaces.  Conventions:
 *   - every call returns a dob_status; no exception or abort crosses the ABI;
 *   - caller-owned host buffers are copied synchronously before the call
 *     returns;
 *   - a context owns all of its device memory and is not re-entrant; separate
 *     contexts may be driven from separate threads;
 *   - grids are x-fastest: index = (z * ny + y) * nx + x.  The MAC faces use
 *     the reference's upper-face convention: u(i,j,k) lives on the +x face of
 *     cell (i,j,k), v on the +y face, w on the +z face
 *     (src/shaders/fluid.ts:96-99).
 */
#ifndef DROPFLUID_H
#define DROPFLUID_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DOB_ABI_VERSION 1

typedef struct dob_ctx dob_ctx;

typedef enum dob_status {
  DOB_OK = 0,
  DOB_EINVAL = -1,       /* bad argument (dims, sizes, pointers, NaN dt ...) */
  DOB_ENOMEM = -2,       /* device or host allocation failed               */
  DOB_ECUDA = -3,        /* a CUDA runtime call failed                      */
  DOB_ENOCONVERGE = -4,  /* pressure solve missed its tolerance             */
  DOB_ETIMEOUT = -5,     /* a bounded device wait ran out                    */
  DOB_ESTATE = -6        /* call not valid in the context's current state   */
} dob_status;

/* Boundary conditions of the pressure problem. */
enum {
  /* Reference: 5 Neumann walls + Dirichlet free-surface top whose ghost
     pressure comes from the wave field and the drop necks
     (src/shaders/fluid.ts:16-77, 561-603). */
  DOB_BC_REFERENCE = 0,
  /* Closed box, free-slip walls, pure Neumann pressure (singular problem:
     FP64 zero-mean compatibility of the right-hand side, pressure mean
     pinned to zero). */
  DOB_BC_CLOSED_BOX = 1
};

/* Storage precision. Arithmetic is FP32 in every mode. */
enum {
  DOB_PREC_FP32 = 0,           /* all fields FP32                                   */
  DOB_PREC_MIXED = 1,          /* FP16 dye; pressure as an FP32 pair (double-float)
                                  corrected by rounds of an error-free residual and
                                  V-cycles on the correction that store levels >= 2
                                  as BF16; needs mg_levels >= 2                      */
  DOB_PREC_REFERENCE_FP16 = 2  /* velocity/curl/dye stored as binary16 like the
                                  reference's rgba16float textures; pressure FP32  */
};

/* Physics terms of the reference step (all on in reference mode). */
enum {
  DOB_PHYS_VORT_CONF = 1,      /* vorticity confinement (fluid.ts:401-423, 467-472)   */
  DOB_PHYS_BUOYANCY = 2,       /* Boussinesq buoyancy on y faces (fluid.ts:474-486)   */
  DOB_PHYS_SPONGE = 4,         /* circular sponge + floor layer (fluid.ts:312-321)    */
  DOB_PHYS_NECK = 8,           /* drop-neck momentum blend (fluid.ts:198-285)         */
  DOB_PHYS_SOLENOIDAL = 16,    /* deep-column solenoidal forcing (fluid.ts:488-503)   */
  DOB_PHYS_SURFACE = 32,       /* Marangoni + kinematic top layers (fluid.ts:287-310) */
  DOB_PHYS_REFERENCE_ALL = 63,
  DOB_PHYS_WAVE = 64,          /* run the 512x512 wave solver (wave.ts:55-388) at the start
                                  of every step, before the advection (BloodDropEngine.ts:
                                  1886-1912); without it the wave field is an input      */
  DOB_PHYS_LIGHTING = 128      /* end every dob_step / dob_step_uniforms call with the light
                                  volume and brick passes (dob_light_volume), as the
                                  reference's frame encodes them once after its substeps
                                  (BloodDropEngine.ts:2601-2616, 2629-2664)              */
};

/* Step configuration (plain data, versioned by struct_size). */
typedef struct dob_config {
  uint32_t struct_size;        /* = sizeof(dob_config)                              */
  uint32_t nx, ny, nz;         /* velocity / pressure grid                           */
  uint32_t dye_refine;         /* 1: dye on the velocity grid; 2: 2x super-resolved
                                  dye grid (reference: 192x256x192 over 96x128x96)   */
  float dx;                    /* closed-box cell size (world units)                 */
  float dt;                    /* closed-box time step (reference mode reads dt from
                                  the uniform block, clamped to [0, 0.025])          */
  float domain_min[3];         /* closed-box world box; reference mode takes it from */
  float domain_max[3];         /* the uniform block's domainBounds                  */
  int32_t bc_mode;             /* DOB_BC_*                                           */
  int32_t precision_mode;      /* DOB_PREC_*                                         */
  int32_t mg_levels;           /* grids in the hierarchy (reference: 4); nx, ny, nz
                                  must be divisible by 2^mg_levels so that every grid
                                  has even dims                                      */
  int32_t mg_pre, mg_post;     /* RBGS sweeps before/after coarse correction          */
  int32_t mg_coarse_sweeps;    /* RBGS sweeps on the coarsest grid (reference: 6);
                                  -1: exact solve with a dense (pseudo-)inverse,
                                  coarsest grid of at most 4096 cells              */
  int32_t mg_cycles;           /* V-cycles per step (reference: 1); mixed mode: the
                                  V-cycles the first round of a step runs before
                                  its first convergence test (0: test from the
                                  first cycle on)                                    */
  int32_t mg_max_outer;        /* mixed mode: rounds of defect correction per step
                                  (one error-free residual of the pressure each, then
                                  up to 16 V-cycles on the correction, tested after
                                  each finest-level pre-smoothing); at most 4 are
                                  run, 1..32 accepted                                */
  double mg_rel_tol;           /* mixed mode: stop at ||b-Ap||/||b|| <= this (0: off)  */
  double mg_div_tol;           /* mixed mode: stop at max |b-Ap| (= the projected max
                                  |div u|) scaled like dob_step_stats.max_div <= this
                                  (0: off); both targets must hold                  */
  float casson_tau_y;          /* closed-box Casson yield stress                      */
  float casson_mu_p;           /* closed-box Casson plastic viscosity                 */
  int32_t physics_flags;       /* DOB_PHYS_*                                          */
  uint32_t parcel_capacity;    /* parcel ring size (reference: 393216)               */
  int32_t reference_schedule;  /* 1: L0 uses 1+1 sweeps, coarser levels mg_pre/mg_post,
                                  exactly the reference's V-cycle (BloodDropEngine.ts:
                                  1942-2059); 0: mg_pre/mg_post on every level       */
  float vel_damping;           /* closed box: per-step advection damping (1 = none)   */
  float dye_sharpness;         /* closed box: MacCormack correction strength          */
  int32_t mg_cycles_injected;  /* closed box, FP32/FP16 storage: V-cycles of the first
                                  two steps after dob_inject_sphere /
                                  dob_inject_sphere_soft (a new divergent source the
                                  warm start knows nothing about); 0: mg_cycles.
                                  dob_config_closed_box sets 2 x mg_cycles.
                                  dob_tape_forward runs every recorded step with
                                  mg_cycles.                                           */
} dob_config;

/* Field identifiers for dob_set_field / dob_get_field.  Host data is always
   FP32 (float) except the splat accumulators (uint32).  Sizes in elements:
     VEL_U/V/W, PRESSURE, RHS, DIVERGENCE : nx*ny*nz
     VEL_CENTER, CURL                     : 4*nx*ny*nz (x,y,z,w interleaved)
     CONC    (reference mode)             : 4*Nc   (r,g,b,a interleaved)
     CONC    (closed box: single dye)     : Nc
     CONC_PRED                            : Nc
     SPLAT_INTACT, SPLAT_LYSED            : Nc (uint32)
     WAVE                                 : 4*512*512 (eta, deta/dt, lap, film)
     LIGHT   (reference mode, read-only)  : 4*nx*ny*nz (key light, back light,
                                            multiple scattering, filtered total
                                            haemoglobin), binary16 values
     BRICKS, BRICKS_RAW (reference mode,
             read-only)                   : (nx/4)*(ny/4)*(nz/4)
   with Nc = (dye_refine*nx)*(dye_refine*ny)*(dye_refine*nz). */
typedef enum dob_field {
  DOB_FIELD_VEL_U = 0,
  DOB_FIELD_VEL_V = 1,
  DOB_FIELD_VEL_W = 2,
  DOB_FIELD_VEL_CENTER = 3,
  DOB_FIELD_CURL = 4,
  DOB_FIELD_PRESSURE = 5,
  DOB_FIELD_RHS = 6,
  DOB_FIELD_CONC = 7,
  DOB_FIELD_CONC_PRED = 8,
  DOB_FIELD_SPLAT_INTACT = 9,
  DOB_FIELD_SPLAT_LYSED = 10,
  DOB_FIELD_WAVE = 11,
  DOB_FIELD_DIVERGENCE = 12,   /* read-only: MAC divergence of the current velocity */
  DOB_FIELD_LIGHT = 13,        /* read-only: light volume (lighting.ts:19-170)        */
  DOB_FIELD_BRICKS = 14,       /* read-only: dilated brick occupancy 0/1/2 (lighting.ts:
                                  205-240)                                             */
  DOB_FIELD_BRICKS_RAW = 15,   /* read-only: raw brick occupancy 0/1 (lighting.ts:172-203) */
  DOB_FIELD_COUNT = 16,
  /* Adjoint fields (closed box, FP32 or mixed, dye_refine 1; see
     dob_adjoint_stage).
     Host FP32, natural layout.  ADJ_VEL_U/V/W: adjoint of the MAC faces a
     stage reads (after dob_tape_backward: d loss / d initial velocity);
     ADJ_VEL_U2/V2/W2: adjoint of the faces advection / Casson write to
     their second buffer; ADJ_CENTER: 4*nx*ny*nz (x, y, z, 0); ADJ_CONC
     (after dob_tape_backward: d loss / d initial dye), ADJ_CONC2 (adjoint
     of the resolved dye), ADJ_PRED: Nc; ADJ_PRESSURE, ADJ_RHS: nx*ny*nz. */
  DOB_FIELD_ADJ_VEL_U = 16,
  DOB_FIELD_ADJ_VEL_V = 17,
  DOB_FIELD_ADJ_VEL_W = 18,
  DOB_FIELD_ADJ_VEL_U2 = 19,
  DOB_FIELD_ADJ_VEL_V2 = 20,
  DOB_FIELD_ADJ_VEL_W2 = 21,
  DOB_FIELD_ADJ_CENTER = 22,
  DOB_FIELD_ADJ_CONC = 23,
  DOB_FIELD_ADJ_CONC2 = 24,
  DOB_FIELD_ADJ_PRED = 25,
  DOB_FIELD_ADJ_PRESSURE = 26,
  DOB_FIELD_ADJ_RHS = 27
} dob_field;

/* Stages of one step, in the reference's order (BloodDropEngine.ts:1855-2111).
   dob_run_stage runs exactly one of them on the current state. */
typedef enum dob_stage {
  DOB_STAGE_ADVECT_MAC = 0,      /* FLUID_ADVECT_MAC      fluid.ts:144-329  */
  DOB_STAGE_MAC_TO_CENTER = 1,   /* FLUID_MAC_TO_CENTER   fluid.ts:917-962  */
  DOB_STAGE_CURL = 2,            /* FLUID_CURL            fluid.ts:331-369  */
  DOB_STAGE_CASSON_FORCES = 3,   /* FLUID_CASSON_FORCES   fluid.ts:377-511  */
  DOB_STAGE_MAC_RHS = 4,         /* FLUID_MAC_RHS         fluid.ts:517-555  */
  DOB_STAGE_PRESSURE_SOLVE = 5,  /* V-cycle schedule      BloodDropEngine.ts:1942-2059 */
  DOB_STAGE_PROJECT = 6,         /* FLUID_MAC_PROJECT     fluid.ts:863-911  */
  DOB_STAGE_CLEAR_SPLATS = 7,    /* clearBuffer x2        BloodDropEngine.ts:2074-2075 */
  DOB_STAGE_PARCEL_EMIT = 8,     /* PARTICLE_EMIT         particles.ts:53-181 */
  DOB_STAGE_PARCEL_ADVECT = 9,   /* PARTICLE_ADVECT_SPLAT particles.ts:189-462 */
  DOB_STAGE_CONC_PREDICT = 10,   /* CONC_PREDICT          advect.ts:28-72    */
  DOB_STAGE_CONC_RESOLVE = 11,   /* CONC_RESOLVE          advect.ts:81-298   */
  DOB_STAGE_COUNT = 12
} dob_stage;

/* Flags for dob_step. */
enum {
  DOB_STEP_STATS = 1,   /* fill residual norms, max divergence, parcels alive  */
  DOB_STEP_TIMING = 2,  /* per-stage device milliseconds (runs without a graph) */
  DOB_STEP_NO_GRAPH = 4 /* launch stage by stage instead of replaying a graph   */
};

typedef struct dob_step_stats {
  uint32_t struct_size;
  int32_t steps_done;
  int32_t vcycles;              /* V-cycles in the last step                      */
  int32_t outer_iters;          /* defect-correction iterations in the last step  */
  double rhs_l2;                /* ||b|| of the last pressure solve (FP64)        */
  double residual_l2;           /* ||b - A p|| after the last solve (FP64); -1
                                   when not formed (dob_set_step_stats)         */
  double max_div;               /* max |div u| * dt / dx after projection         */
  uint32_t parcels_alive;       /* 0 when not formed (dob_set_step_stats)         */
  uint32_t pad;
  float stage_ms[DOB_STAGE_COUNT];
} dob_step_stats;

/* ---- lifecycle (replaces BloodDropEngine.create / destroy,
        BloodDropEngine.ts:336-391, 2671-2736) ---------------------------- */

/* Fill *cfg with the reference's own setup: 96x128x96 velocity grid, 2x dye,
   Dirichlet top, 4-grid V-cycle with the reference schedule, 393216 parcels
   (src/shaders/common.ts:4-20; BloodDropEngine.ts:88-98). */
dob_status dob_config_reference(dob_config* cfg);
/* Fill *cfg with a closed-box synthetic scene of the given grid:
   FP32, 2+2 RBGS on every level, 4 cycles, the hierarchy deepened (even dims
   on every grid) until the coarsest grid has at most 2304 cells, solved
   exactly (mg_coarse_sweeps = -1); Casson tau_y=0.005, mu_p=1e-3, dx=1,
   dt=0.02; mixed mode: stop at max |div| dt/dx <= 1e-5, <= 16 iterations. */
dob_status dob_config_closed_box(dob_config* cfg, uint32_t nx, uint32_t ny, uint32_t nz);

dob_status dob_create(const dob_config* cfg, dob_ctx** out);
void dob_destroy(dob_ctx* ctx);
/* Last error message of this context (static string if ctx is NULL). */
const char* dob_last_error(const dob_ctx* ctx);
int dob_abi_version(void);

/* ---- state (replaces resetSimulation, BloodDropEngine.ts:1682-1763) ---- */

/* Reference mode: FLUID_INIT_VEL on both velocity buffers, center and curl
   (seed = uniform globalSeed), pressure/MG/conc/parcels/splats cleared.
   Closed box: fluid at rest, everything zero. */
dob_status dob_reset(dob_ctx* ctx);

/* The reference's 512-byte SimUniforms block, verbatim (common.ts:26-43,
   uniformLayout.ts:56-190).  Used by every following reference-mode step. */
dob_status dob_set_uniforms(dob_ctx* ctx, const float sim_uniforms[128]);

/* Closed box: a sphere of dye `dye` and face velocity vel (world units) plus
   N(0, noise_sigma) noise per face (seeded SplitMix64 + Box-Muller). */
dob_status dob_inject_sphere(dob_ctx* ctx, const float center[3], float radius,
                             float dye, const float vel[3], float noise_sigma,
                             uint64_t seed);

/* Closed box, no counterpart in the reference: a soft-edged drop added to
   the fields.  Weight w = 1 within radius - edge/2 of the centre, 0 beyond
   radius + edge/2, smoothstep in between (continuously differentiable in the
   centre); dye += w dye on the dye grid and each MAC face += w (vel +
   N(0, noise_sigma) noise).  Additive, so its derivative in the drop's
   parameters does not depend on the state it is added to
   (dob_adjoint_sphere_soft).  edge > 0. */
dob_status dob_inject_sphere_soft(dob_ctx* ctx, const float center[3], float radius, float edge,
                                  float dye, const float vel[3], float noise_sigma, uint64_t seed);

/* Parcels: AoS, 8 floats (32 B) each = RbcParcel (particles.ts:17-20).
   dob_set_parcels writes n parcels at ring index `offset` and raises the
   high-water mark; dob_get_parcels reads n parcels from `offset`. */
dob_status dob_set_parcels(dob_ctx* ctx, const float* parcels, uint32_t n, uint32_t offset);
dob_status dob_get_parcels(dob_ctx* ctx, float* parcels, uint32_t n, uint32_t offset);
dob_status dob_set_high_water(dob_ctx* ctx, uint32_t high_water);

dob_status dob_set_field(dob_ctx* ctx, int field, const void* host, size_t bytes);
dob_status dob_get_field(dob_ctx* ctx, int field, void* host, size_t bytes);

/* ---- stepping (replaces encodePhysicsStep / seekToSimTime,
        BloodDropEngine.ts:1855-2111, 2142-2179) ------------------------- */

/* Run nsteps full steps with the current uniform block.  `stats` may be
   NULL.  In reference mode the spawn count and cursor come from the uniform
   block (particleParams.y/.z) and the high-water mark advances by the spawn
   count like BloodDropEngine.ts:1832-1840. */
dob_status dob_step(dob_ctx* ctx, int nsteps, uint32_t flags, dob_step_stats* stats);

/* Pipelined stepping: dob_step_async enqueues one step with statistics
   (as DOB_STEP_STATS) whose results land in pinned result slot `slot`
   (0..7) and returns without waiting; dob_step_result waits for that step
   and fills *stats.  Keeping one or two steps in flight hides the host's
   wait behind the next step's device work (the reference reads its GPU
   timestamps back asynchronously the same way, BloodDropEngine.ts:2400-2456).
   A slot must be read back before it is reused. */
dob_status dob_step_async(dob_ctx* ctx, int slot);
dob_status dob_step_result(dob_ctx* ctx, int slot, dob_step_stats* stats);

/* Which statistics a step with DOB_STEP_STATS (and dob_step_async) forms.
   max |div| and ||b|| always (in the closed box they come out of the
   projection and the mean removal at no extra pass; in reference mode they
   are a divergence pass and a sum of squares).  DOB_STATS_RESIDUAL adds
   ||b - A p|| (one
   error-free residual pass over the pressure, about 60 us at 192x256x192),
   DOB_STATS_PARCELS the live-parcel count (one reduction over the ring).
   Default DOB_STATS_ALL; the fields of a step are the same bits whatever
   the mask.  (The reference reads back only GPU timestamps per frame,
   BloodDropEngine.ts:2400-2456.) */
#define DOB_STATS_RESIDUAL 1u
#define DOB_STATS_PARCELS 2u
#define DOB_STATS_ALL 3u
dob_status dob_set_step_stats(dob_ctx* ctx, uint32_t mask);

/* Reference mode: nsteps substeps, each with its own 128-float block
   (the reference's multi-substep staging path, BloodDropEngine.ts:2634-2651). */
dob_status dob_step_uniforms(dob_ctx* ctx, const float* blocks, int nsteps,
                             uint32_t flags, dob_step_stats* stats);

/* Run exactly one stage of the step on the current state (parity tests). */
dob_status dob_run_stage(dob_ctx* ctx, int stage);
/* One substep of the 512x512 gravity-capillary wave solver on the wave field
   (DOB_FIELD_WAVE), from the current uniforms and v faces: replaces the
   seven wave passes of encodePhysicsStep (wave.ts:55-388,
   BloodDropEngine.ts:1886-1912).  dob_step runs it at the start of every
   step when the context was created with DOB_PHYS_WAVE in reference mode;
   DOB_ESTATE otherwise. */
dob_status dob_wave_step(dob_ctx* ctx);

/* The light volume and the empty-space brick map from the current dye and
   wave fields and uniform block: replaces encodeLightingPasses
   (lighting.ts:19-240; BloodDropEngine.ts dispatches it after each frame's
   physics and at the reset).  Per velocity-grid voxel: key-light
   transmittance with wave caustics and drop shadows, back-light
   transmittance, multiply scattered red light, filtered total haemoglobin,
   stored as binary16 (rgba16float); then the 4x4x4 brick occupancy of the
   filtered total and its two-shell dilation.  Reference mode with nx, ny,
   nz divisible by 4 (DOB_ESTATE otherwise).  Queued on the context's
   stream; dob_reset runs it too. */
dob_status dob_light_volume(dob_ctx* ctx);

/* Device time of nsteps steps (dob_step with `flags`; with DOB_STEP_STATS
   the statistics kernels run but nothing is read back), measured with CUDA
   events on the context's stream; replaces the reference's per-pass GPU
   timestamp queries (BloodDropEngine.ts:2400-2456). */
dob_status dob_time_steps(dob_ctx* ctx, int nsteps, uint32_t flags, float* ms);

/* Kernel micro-benchmark on the current state: launches the step's dominant
   kernel (which = 0: the level-0 pressure smoother pass; which = 1: one
   wave substep, its four kernels, on a context made with DOB_PHYS_WAVE;
   which = 2: the light volume and brick passes, reference mode; which = 3:
   the plume march at the last dob_render_plume's size) `reps` times with
   CUDA events around each launch; returns the mean device ms per launch and
   the kernel's algorithmic bytes per launch (minimum HBM traffic of one
   pass).  No counterpart in the reference. */
dob_status dob_bench_kernel(dob_ctx* ctx, int which, int reps, float* avg_ms, double* bytes_per_launch);

/* Block until all queued device work of this context is done. */
dob_status dob_sync(dob_ctx* ctx);

/* Kernels launched by one step (kernel nodes of the captured step graph). */
dob_status dob_launches_per_step(dob_ctx* ctx, int* n);

/* Host<->device bytes of one step through this ABI: the per-step parameter
   block copied host->device before each step, and the statistics read back
   device->host by a dob_step with DOB_STEP_STATS. */
dob_status dob_io_bytes(const dob_ctx* ctx, uint64_t* h2d_per_step, uint64_t* d2h_stats);

/* Device memory held by this context, in bytes. */
dob_status dob_memory_bytes(const dob_ctx* ctx, uint64_t* bytes);

/* Copy of the whole simulation state into snapshot slot 0..7 (device memory)
   and back.  Slots are allocated on first use. */
dob_status dob_save_state(dob_ctx* ctx, int slot);
dob_status dob_load_state(dob_ctx* ctx, int slot);

/* ---- plume render (render.ts:1593-2109, 2411-2434, 2659-2688) -----------

   The volumetric plume march of the reference renderer (marchPlume) as a
   headless image: per pixel fsMain's camera ray and thin lens from the
   uniform block (invViewProj, camera position, focal distance, aperture,
   frame index for the jitter), driven as the submerged camera's primary
   march from 0.02 to the meniscus (rays steeper than 0.052 upward end
   where they cross the wave surface, intersectWaterSurface, render.ts:
   1004-1128; the others at the flat plane), with the reference's
   constants, fine quality and the inspect mode off.  Reference
   mode with nx, ny, nz divisible by 4.

   dob_set_spectral_lut stores the renderer's 256 x 64 spectral
   transmittance table (the reference builds it on the host and uploads it
   as an rgba texture: u = tau / (0.012 + 0.996 tau), v = oxygenated
   fraction); host FP32, 4 floats (r, g, b, a) per texel, row-major, u
   fastest.

   dob_render_plume computes the light volume of the current state (the
   frame's lighting pass, as dob_light_volume) and then, per pixel of a
   width x height image (y down, pixel centres), 8 binary16 values: the
   plume's radiance r, g, b, its total optical depth, its transmittance r,
   g, b and its intact-cell optical depth; the composite is behind *
   transmittance + radiance (render.ts:2632).  out: host, bytes = width x
   height x 16.  Blocks until the image is on the host. */
#define DOB_SPECTRAL_LUT_W 256
#define DOB_SPECTRAL_LUT_H 64
dob_status dob_set_spectral_lut(dob_ctx* ctx, const float* rgba, size_t bytes);
dob_status dob_render_plume(dob_ctx* ctx, uint32_t width, uint32_t height, uint16_t* out, size_t bytes);

/* ---- discrete adjoint (no counterpart in the reference; closed box, FP32
        or DOB_PREC_MIXED, dye_refine 1) -----------------------------------

   dob_adjoint_stage runs the transpose of the Jacobian of one stage at the
   current forward state (the state the forward stage would read), on the
   adjoint fields:
     ADVECT_MAC      ADJ_VEL_*2 -> ADJ_VEL_*, ADJ_CENTER   (accumulate)
     MAC_TO_CENTER   ADJ_CENTER -> ADJ_VEL_*
     CASSON_FORCES   ADJ_VEL_*2 -> ADJ_VEL_*, ADJ_CONC
     MAC_RHS         ADJ_RHS -> ADJ_VEL_* (ADJ_RHS is made mean-free in place)
     PRESSURE_SOLVE  ADJ_PRESSURE -> ADJ_PRESSURE (replaced), ADJ_RHS
                     FP32: the transpose of the mg_cycles V-cycles (the
                     replaced ADJ_PRESSURE is the adjoint of the warm start);
                     mixed: the forward is solved to a tolerance, so its
                     adjoint is that of an exact solve: ADJ_RHS += lam with
                     A lam = ADJ_PRESSURE solved by the mixed solver to a
                     relative residual of 1e-6, ADJ_PRESSURE set to 0
     PROJECT         ADJ_VEL_* -> ADJ_VEL_* (replaced), ADJ_PRESSURE
     CONC_PREDICT    ADJ_PRED -> ADJ_CONC, ADJ_CENTER
     CONC_RESOLVE    ADJ_CONC2 -> ADJ_CONC, ADJ_PRED, ADJ_CENTER
   Other stages return DOB_EINVAL.  Where the forward is not differentiable
   (clamps at their bounds, the dye limiter, |grad u| = 0) the adjoint takes
   the branch the forward executed.  In the mixed mode the dye and the
   predictor are read at their binary16 values (the adjoint of a rounding
   store is the identity); the adjoint fields stay FP32. */
dob_status dob_adjoint_stage(dob_ctx* ctx, int stage);

/* Forward half of the forward/backward pair: sets the centre velocity from
   the MAC faces (so the trajectory's state is velocity, dye and pressure),
   then runs nsteps steps, keeping a checkpoint of (velocity, dye, pressure)
   every `checkpoint_every` steps in device memory (mixed mode: the dye at
   its binary16 width and the pressure as its FP32 pair).  The steps of the last
   segment also record the linearisation points the backward needs, so the
   next dob_tape_backward does not recompute that segment; with
   checkpoint_every = nsteps that is the whole trajectory (the tape then
   holds nsteps steps' points, about 0.45 GB per step at 192x256x192 in
   FP32).  The context ends in the final state, as after dob_step (same
   bits). */
dob_status dob_tape_forward(dob_ctx* ctx, int nsteps, int checkpoint_every);

/* Backward half: given d loss / d final dye (Nc floats, host), recomputes
   each checkpoint segment (all but the last after dob_tape_forward; every
   one when called again) and runs the adjoint of every step in reverse.
   Leaves d loss / d initial MAC velocity in DOB_FIELD_ADJ_VEL_U/V/W,
   d loss / d initial dye in DOB_FIELD_ADJ_CONC and d loss / d initial
   pressure in DOB_FIELD_ADJ_PRESSURE.  The forward state is not changed. */
dob_status dob_tape_backward(dob_ctx* ctx, const float* dye_grad, size_t bytes);

/* Sum over the MAC faces dob_inject_sphere(center, radius, ..) sets of
   ADJ_VEL . vel: d loss / d s when the injected face velocity is s * vel
   (+ noise). */
dob_status dob_adjoint_sphere_impulse(dob_ctx* ctx, const float center[3], float radius, const float vel[3],
                                      double* out);

/* Gradient of the loss in the parameters of a dob_inject_sphere_soft drop
   (same arguments) from the adjoint fields DOB_FIELD_ADJ_VEL_U/V/W and
   DOB_FIELD_ADJ_CONC of the state right after the drop (after
   dob_tape_backward: the trajectory's initial state).  out[0] = d loss / d s
   for injected velocity s * vel at s = 1 (the noise is not scaled); out[1..3]
   = d loss / d center (world units).  Closed box, FP32 or mixed, dye_refine 1. */
dob_status dob_adjoint_sphere_soft(dob_ctx* ctx, const float center[3], float radius, float edge, float dye,
                                   const float vel[3], float noise_sigma, uint64_t seed, double out[4]);

/* Evaluate the library's own elementary functions on the device (used to
   check them against the host build bit for bit).  fn: 0 sin, 1 cos, 2 exp,
   3 log, 4 pow(x,y), 5 atan2(x,y), 6 tanh, 7 f32->f16->f32 round trip,
   8 f32->bf16->f32 round trip, 9 x / y as the kernels divide by a launch
   constant (the correctly rounded reciprocal and one remainder correction:
   the IEEE quotient). */
dob_status dob_eval_math(int fn, const float* x, const float* y, float* out, uint32_t n);

/* ---- pressure solve without allocation (no counterpart in the reference) --

   The multigrid pressure solve of one step (the same V-cycles as
   DOB_STAGE_PRESSURE_SOLVE, including the zero-mean pressure of the closed
   box) on caller-owned device buffers, for callers that cannot allocate
   device memory: hosts whose own allocator owns the whole GPU, plugins
   running inside such hosts, and frame loops that must not call cudaMalloc
   or cudaFree (both synchronise the device and can fail mid-frame).  No
   context is needed and nothing is allocated: the working arrays (split
   copies, coarse grids, reduction slots) live in one fixed device array of
   about 40 MiB that is part of the library and stays resident on every GPU
   that loads it until the process exits.

   rhs and pressure are device pointers of the current device, nx*ny*nz
   floats each in the natural x-fastest layout; pressure is the initial
   guess on entry and the solution on return.  From cfg only nx, ny, nz,
   bc_mode, precision_mode (DOB_PREC_FP32 or DOB_PREC_REFERENCE_FP16; the
   pressure is FP32 in both), mg_levels, mg_pre, mg_post, mg_coarse_sweeps,
   mg_cycles and reference_schedule are read.  At most 2^21 cells
   (2097152, e.g. 96x128x96 or 128^3): larger grids return DOB_EINVAL, and
   so does an exact coarsest solve (mg_coarse_sweeps = -1) on a coarsest
   grid of more than 2304 cells.
   The work is queued on `stream` (a cudaStream_t; NULL is the default
   stream) and the call returns without waiting for it.

   Every call shares the one array and leaves its contents there: calls whose
   work overlaps on the GPU (unordered streams, concurrent host threads)
   race; order them on one stream.  The first call on each device performs a
   one-time set-up with that device current (cudaGetSymbolAddress of the
   array, the coarse-grid kernel's shared-memory limit); make it before any
   stream capture.  With an exact coarsest solve, a call whose coarsest grid
   differs from the previous such call's on this device (dims, bc_mode, or
   mg_levels relative to the fine grid, which sets the coarse spacing)
   rebuilds the grid's dense inverse on the host and uploads it into the
   array: that call waits for `stream` to drain before it returns and must
   not be made during stream capture.  Errors: dob_last_error(NULL). */
dob_status dob_pressure_solve_noalloc(const dob_config* cfg, const float* rhs, float* pressure, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* DROPFLUID_H */
