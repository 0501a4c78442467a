/*
 * dcg.h — C ABI of the GB300-native DCGrid simulation step.
 *
 * This header replaces the reference's C++ simulation interface
 *   FluidSimulation (src/fluid_simulation.h:4-27),
 *   FluidSimulationDCGrid(const int3&, const size_t&)  (src/dcgrid/fluid_simulation_dcgrid.h:7),
 *   FluidSimulationUniform(const int3&)                 (src/uniformgrid/fluid_simulation_uniform.h:7),
 *   copySimParamsToDevice(SimParams&)                   (src/utils/sim_utils.h:5-6)
 * with plain functions over an opaque handle. Every call returns an int status
 * (DCG_OK or a DCG_E_* code) instead of calling exit(1) as the reference does
 * (src/dcgrid/fluid_simulation_dcgrid.cu:35-53, include/cuda/helper_cuda.h:761-790).
 *
 * Threading: one handle is not thread-safe; separate handles are independent.
 * All device work of a handle is issued on that handle's CUDA stream.
 */
#ifndef DCG_H
#define DCG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
enum {
  DCG_OK = 0,
  DCG_E_INVALID = 1,   /* bad argument / unsupported configuration            */
  DCG_E_BUDGET = 2,    /* block budget cannot hold the coarsest level or L0   */
  DCG_E_HASH_FULL = 3, /* reserved: no hash exists in this implementation     */
  DCG_E_CUDA = 4,      /* a CUDA runtime call failed                          */
  DCG_E_TIMEOUT = 5,   /* a bounded device-side wait gave up                  */
  DCG_E_NAN = 6,       /* a non-finite value was produced                     */
  DCG_E_NOT_FOUND = 7, /* no such field / handle state                        */
  DCG_E_DEVICE = 8     /* device-side error word was set (see error string)   */
};

/* ---- grid type (the reference's adaptive/uniform switch,
 *      src/simulation.cpp:32-35,52-64) -------------------------------------- */
enum { DCG_MODE_ADAPTIVE = 0, DCG_MODE_UNIFORM = 1 };

/* ---- solids / scene SDF (src/sdf.cuh:8-20, src/utils/sim_utils.cu:11-22) - */
enum {
  DCG_SOLIDS_NONE = 0,    /* enable_additional_solids = false                */
  DCG_SOLIDS_SPHERE = 1,  /* the reference's sphere obstacle                 */
  DCG_SOLIDS_TERRAIN = 2, /* extension: heightfield terrain, y - h(x,z)      */
  DCG_SOLIDS_BOTH = 3
};

/* ---- refinement criterion --------------------------------------------- */
enum {
  DCG_REFINE_GEOMETRIC = 0, /* src/dcgrid/dcgrid_adaptation.cu:26-34          */
  DCG_REFINE_FIELDS = 1     /* extension: |curl v| and |grad rho| thresholds */
};

/* ---- storage precision of the advected scalars ------------------------
 * Scalars (density, temperature, vapor) are stored in the given format and
 * computed in FP32; velocity, pressure and fluidity stay FP32. Conversions
 * round to nearest even. */
enum {
  DCG_PRECISION_FP32 = 0,
  DCG_PRECISION_MIXED = 1,      /* BF16 scalars */
  DCG_PRECISION_MIXED_FP16 = 2  /* FP16 scalars */
};

/*
 * Simulation parameters. Units follow the reference's SimParams
 * (src/data/sim_params.h:14-47): positions in finest-level cells, velocities in
 * world units per time unit, dx = world size of one finest cell (rdx = 1/dx).
 * Unlike the reference's single __constant__ SimParams, every handle owns its
 * own copy, so simulations in one process may differ.
 */
typedef struct dcg_params {
  int32_t gx, gy, gz;    /* domain size in finest cells                      */
  int32_t levels;        /* 0 = derive as the reference does (cu:12-22)      */
  int64_t max_blocks;    /* block budget (the reference's maxNumBlocks)      */
  float dt;              /* time step                                        */
  float dx;              /* world size of a finest cell                      */

  /* reference inlet BC (src/utils/sim_utils.cu:24-55) */
  int32_t inlet_enabled;
  float velocity_emission_rate;
  float density_emission_rate;
  float emission_radius; /* world units                                      */

  /* solids / fluidity */
  int32_t solids;            /* DCG_SOLIDS_*                                 */
  float sphere_radius_world; /* reference: 2000 world units (sdf.cuh:12)     */

  /* solver */
  int32_t jacobi_iters;      /* sweeps per level; reference: 10 (5 pairs)    */
  int32_t init_adapt_passes; /* reference: 5 (fluid_simulation_dcgrid.cu:207) */

  /* adaptation */
  int32_t refine_criterion;  /* DCG_REFINE_*                                 */
  float refine_threshold;    /* reference: 1e-4 (cu:461)                     */
  float vort_threshold;      /* extension: |curl v| scale                    */
  float grad_threshold;      /* extension: |grad rho| scale                  */
  int32_t ref_compat;        /* 1 = reproduce the reference's selection quirks */

  /* extension: scalars, buoyancy, sources, wind */
  int32_t n_scalars;         /* 1 = density (reference); 3 = density, temperature, vapor */
  float buoy_alpha, buoy_beta, t_ambient;
  int32_t src_enabled;       /* sphere source, values set every step          */
  float src_center[3];       /* finest cells                                 */
  float src_radius;          /* finest cells                                 */
  float src_density, src_temperature, src_vapor;
  int32_t wind_enabled;      /* inflow at x<0, zero-gradient outflow at x>=gx */
  float wind[3];             /* world units per time unit                     */

  /* extension: terrain SDF from seeded value noise */
  float terrain_amplitude;   /* finest cells                                 */
  float terrain_base_height; /* finest cells                                 */
  float terrain_frequency;   /* lattice frequency of the first octave, 1/cells */
  float terrain_persistence;
  int32_t terrain_octaves;
  uint32_t terrain_seed;

  int32_t precision;         /* DCG_PRECISION_*                              */

  /* extension: an emission_n^3 density-emission field (set with
   * dcg_set_emission) spanning x, z and the bottom emission_band cells in y;
   * leaf cells there gain dt * E(trilinear) of density every step. */
  int32_t emission_n;        /* 0 = no emission field                        */
  float emission_band;       /* finest cells                                 */
  /* extension: seeded per-cell jitter of the source temperature, src_temperature
   * + src_jitter * u with u in [-1, 1) from the cell's level-local position */
  float src_jitter;
  uint32_t src_jitter_seed;
  /* extension: FP64 defect correction of the pressure solve. After the
   * cascade, each pass computes the residual r = div - A p of every level's
   * Jacobi equation in FP64 (with FP64 norms), solves A e = r with the same
   * FP32 cascade, and adds e to p. 0 = the reference's cascade alone.
   * Adaptive grid, single simulations. */
  int32_t defect_passes;
  int32_t reserved[3];
} dcg_params;

/* Fills *p with the reference's defaults (src/data/sim_params.cpp:4-34) for a
 * gx*gy*gz domain and the reference's solver/adaptation constants. */
void dcg_default_params(dcg_params *p, int32_t gx, int32_t gy, int32_t gz,
                        int64_t max_blocks);

/* ---- fields ------------------------------------------------------------ */
enum {
  DCG_FIELD_DENSITY = 0,
  DCG_FIELD_VEL_X = 1,
  DCG_FIELD_VEL_Y = 2,
  DCG_FIELD_VEL_Z = 3,
  DCG_FIELD_FLUIDITY = 4,
  DCG_FIELD_PRESSURE = 5,
  DCG_FIELD_PRESSURE_TMP = 6,
  DCG_FIELD_DIVERGENCE = 7,
  DCG_FIELD_TEMPERATURE = 8,
  DCG_FIELD_VAPOR = 9,
  DCG_FIELD_COUNT = 10
};
enum { DCG_HOST = 0, DCG_DEVICE = 1 };

/* Static description of a handle. Arrays hold up to 16 levels. */
typedef struct dcg_info {
  int32_t mode;
  int32_t levels;
  int32_t sparse_levels;       /* levels [0, sparse_levels) are hashed in the reference */
  int32_t n_scalars;
  int64_t max_blocks;          /* block pool size                               */
  int64_t num_cells;           /* 64 * max_blocks (adaptive) or gx*gy*gz (uniform) */
  int64_t full_blocks[16];     /* blocks that cover the whole domain per level  */
  int64_t budget[16];          /* maxNumBlocksLevel                             */
  int64_t offset[16];          /* levelOffsets                                  */
  int64_t device_bytes;        /* bytes of device memory held by the handle     */
} dcg_info;

/* Per-step counters (the reference's debugStats, cu:517-529, plus more). */
typedef struct dcg_stats {
  int64_t load[16];            /* allocated blocks per level                   */
  int64_t leaf_cells[16];      /* cells whose subblock has no child, per level */
  int64_t active_cells;        /* sum of leaf_cells                             */
  int64_t moved_blocks;        /* by the last adaptation                        */
  int64_t refined_subblocks;   /* by the last adaptation                        */
  int64_t steps;
  double residual;             /* sum scale*|div - lap p| over leaf cells      */
  double mass;                 /* sum rho*fluidity*scale^3 over leaf cells     */
  uint32_t device_error;       /* device error word (DCG_DEVERR_* bits)         */
  uint32_t pad;
  double defect_rel_residual[2]; /* FP64 ||r|| / ||div|| of the last projection's
                                    equations before the first and after the last
                                    defect-correction pass (0 without passes)   */
} dcg_stats;

enum {
  DCG_DEVERR_BUDGET = 1u,      /* a refinement found its level full             */
  DCG_DEVERR_LOOKUP = 2u,      /* a block lookup failed                         */
  DCG_DEVERR_NAN = 4u,
  DCG_DEVERR_TIMEOUT = 8u
};

typedef struct dcg_sim dcg_sim;

/* ---- lifecycle (FluidSimulationDCGrid ctor/dtor/reset/init,
 *      fluid_simulation_dcgrid.cu:9-261; FluidSimulationUniform ctor,
 *      fluid_simulation_uniform.cu:6-54) ------------------------------------ */
int dcg_create(const dcg_params *params, int32_t mode, dcg_sim **out);
int dcg_destroy(dcg_sim *sim);
int dcg_reset(dcg_sim *sim);               /* FluidSimulation::reset (+ init)    */
int dcg_set_params(dcg_sim *sim, const dcg_params *params); /* copySimParamsToDevice;
                                               geometry/budget must not change */
int dcg_set_mode(dcg_sim **sim, int32_t mode); /* the N-key switch: recreate,
                                               state not transferred (simulation.cpp:52-64) */
int dcg_set_stream(dcg_sim *sim, void *cuda_stream);
int dcg_get_info(const dcg_sim *sim, dcg_info *info);
const char *dcg_last_error_string(const dcg_sim *sim);

/* ---- the step and its stages (simulation.cpp:104-112; stage bodies in
 *      fluid_simulation_dcgrid.cu:263-346 and fluid_simulation_uniform.cu:62-142) */
int dcg_step(dcg_sim *sim, int32_t n);     /* n x {advect_velocity, adapt, project, advect_scalars} */
int dcg_advect_velocity(dcg_sim *sim);     /* + buoyancy when enabled                */
int dcg_adapt(dcg_sim *sim);               /* adaptTopology                          */
int dcg_project(dcg_sim *sim);             /* cascadic Jacobi projection             */
int dcg_project_local(dcg_sim *sim);       /* projectLocal                           */
int dcg_advect_scalars(dcg_sim *sim);      /* advectDensity (+ temperature, vapor, sources) */
int dcg_sync(dcg_sim *sim);                /* wait for the handle's stream; read the device error
                                               word: DCG_E_NAN when it holds only DCG_DEVERR_NAN,
                                               DCG_E_DEVICE for any other bit */

/* Sets the emission field (emission_n^3 floats, x fastest) from host or
 * device memory. The copy is ordered on the handle's stream before later
 * steps; the step reads it in place, so it may change between steps. */
int dcg_set_emission(dcg_sim *sim, const float *field, int32_t where);

/* Terrain from a heightmap instead of the seeded value noise (the role of the
 * reference's MipmappedTex::loadFromBuffer, utils/mipmapped_tex.h:64-66, an
 * input its step never reads). heights: nx*nz floats, x fastest, from host or
 * device memory; texel (i, k) sits at x = (i + 0.5)*gx/nx, z = (k + 0.5)*gz/nz
 * in finest cells. The terrain height at (x, z) is terrain_base_height +
 * terrain_amplitude * m, m the bilinear sample of the map (edge texels
 * extended), and enters the SDF and fluidity like the noise terrain
 * (solids must include DCG_SOLIDS_TERRAIN). The scene's solids are part of
 * the initial state, so the call resets the simulation. heights == NULL
 * (nx = nz = 0) returns to the noise terrain, also with a reset. The map is
 * an input, not state: dcg_save_state does not store it, and dcg_set_mode
 * recreates the handle without it. Not for members of a batch. */
int dcg_set_heightmap(dcg_sim *sim, const float *heights, int32_t nx, int32_t nz, int32_t where);

/* Adds seeded uniform noise in [-amplitude, amplitude] to every velocity
 * component of every allocated cell (deterministic counter-based hash). */
int dcg_add_velocity_noise(dcg_sim *sim, uint64_t seed, float amplitude);

/* ---- field and topology access (no counterpart in the reference: fields are
 *      private there, fluid_simulation_dcgrid.h:59-60) ----------------------- */
/* Canonical layout: adaptive = block-major, cell c of block b at b*64 + c with
 * the reference's local order (subblock bits x,y,z then cell bits x,y,z,
 * dcgrid_utils.cuh:69-81); uniform = x-fastest dense array. fp32 only. */
int dcg_get_field(dcg_sim *sim, int32_t field, float *dst, int32_t where);
int dcg_set_field(dcg_sim *sim, int32_t field, const float *src, int32_t where);
/* Dense gx*gy*gz x-fastest resampling: each finest cell takes the value of the
 * leaf cell that covers it. */
int dcg_get_dense(dcg_sim *sim, int32_t field, float *dst, int32_t where);
/* Same result as dcg_get_dense, but the call allocates no device memory.
 * No counterpart in the reference. dcg_get_dense cudaMallocs a staging buffer
 * on its first call; callers that cannot allocate at that moment - hosts that
 * give the library a fixed device-memory budget up front, real-time loops that
 * must not take cudaMalloc's device-wide synchronisation mid-frame - use this
 * variant. It stages through a fixed device array of 2^20 floats (4 MiB, held
 * by every GPU that loads the library until exit), so domains of more than
 * 2^20 finest cells are rejected with DCG_E_INVALID. The handle's device must
 * be current, as for every other call. The first call on a device looks the
 * array up (cudaGetSymbolAddress), so make that first call before any stream
 * capture. All calls on a device share the array: calls that overlap on the
 * GPU (other streams or handles) race. Like dcg_get_dense, the call waits for
 * the handle's stream before it returns. */
int dcg_get_dense_noalloc(dcg_sim *sim, int32_t field, float *dst, int32_t where);

/* Block table, host buffers sized by dcg_info.max_blocks:
 *   pos[4*b] = x, y, z (level-local cells), level (-1 = free)
 *   parent[b] = 8*parentBlock + subblock or 0xFFFFFFFF
 *   child[8*b + s] = child block or 0xFFFFFFFF
 *   flags[b] (1 = moved, 2 = refined by the last adaptation)
 *   load[L], move_limit[L] per level.
 * Any pointer may be NULL. set_topology rebuilds neighbour tables. */
int dcg_get_topology(dcg_sim *sim, int32_t *pos, uint32_t *parent,
                     uint32_t *child, uint8_t *flags, int64_t *load,
                     int64_t *move_limit);
int dcg_set_topology(dcg_sim *sim, const int32_t *pos, const uint32_t *parent,
                     const uint32_t *child, const int64_t *load,
                     const int64_t *move_limit);
/* The reference's 6x6x6 apron index table per block (dcgrid.h:22), derived
 * from the neighbour tables: dst[216*b + 36*i + 6*j + k] = global cell index,
 * -1 for free blocks. Host buffer of 216*max_blocks entries. */
int dcg_get_apron(dcg_sim *sim, int64_t *dst);

/* Decisions of the last dcg_adapt: moves (block, destination subblock) and
 * refinements (subblock, new block) in application order. Counts are returned
 * in *n_moves / *n_refines; buffers may be NULL to query counts only. */
int dcg_get_last_adapt(dcg_sim *sim, int64_t *moves, int64_t *n_moves,
                       int64_t *refines, int64_t *n_refines);

/* Runs the statistics pass (which also flags non-finite values: a NaN or
 * infinity in a leaf cell's pressure, divergence, density or fluidity sets
 * DCG_DEVERR_NAN) and fills *stats; returns DCG_E_NAN, with *stats filled,
 * when the device error word holds DCG_DEVERR_NAN. */
int dcg_get_stats(dcg_sim *sim, dcg_stats *stats);

/* ---- extras without a counterpart in the reference -------------------- */
/* dcg_step replays a captured CUDA graph of the whole step (default on). */
int dcg_set_graphs(dcg_sim *sim, int32_t on);
/* Times `reps` launches of one kernel on the current state with CUDA events
 * on the handle's stream; *avg_ms = mean duration of one launch, *bytes =
 * algorithmic bytes of one launch. which: 0 = Jacobi sweep of `level`,
 * 1 = velocity advection, 2 = scalar advection, 3 = divergence. */
int dcg_time_kernel(dcg_sim *sim, int32_t which, int32_t level, int32_t reps,
                    float *avg_ms, double *bytes);
/* Number of kernel launches one dcg_step performs (kernel nodes of the
 * captured step graph; 0 before the first graph capture). */
int dcg_launches_per_step(dcg_sim *sim, int64_t *n);
/* Self-check of the solver arithmetic on the current device: the Jacobi
 * update divides by six with a multiply and two FMAs (a correctly rounded
 * method for a divisor known in advance) instead of the IEEE division. Runs
 * both over every binary32 input; *mismatches = inputs whose results differ
 * (NaNs compare equal), *first = the smallest such input's bit pattern
 * (0xFFFFFFFF when none). */
int dcg_check_div6(uint64_t *mismatches, uint32_t *first);
/* Self-check of the bounded device-side waits (no reference counterpart; the
 * reference has no grid-wide waits). Launches, on the handle's stream, a
 * two-CTA cooperative kernel in which one CTA never arrives at the grid
 * barrier that the level solves use: the other gives up after poll_limit
 * polls (1 .. 2^20; the solves use 2^22) and sets DCG_DEVERR_TIMEOUT in the
 * handle's device error word, so the next dcg_sync returns DCG_E_DEVICE.
 * Nothing hangs and the context stays usable; dcg_reset clears the word.
 * Adaptive handles that are not batch members. */
int dcg_check_barrier_timeout(dcg_sim *sim, uint32_t poll_limit);
/* ---- batches: many independent adaptive simulations stepped together -----
 * No reference counterpart: the reference runs one simulation per process
 * (one global __constant__ parameter set, src/utils/sim_utils.h:5-6). A batch
 * owns n adaptive simulations with their own parameters, domains, level
 * counts and budgets; every field stage of a batch step is one launch over
 * all members (groups of 16 members per launch), each cascade round of the
 * pressure solve is one cooperative launch over the members' cells, the
 * members' adaptations run as parallel branches, and the whole step is one
 * CUDA graph. A member's results equal those of a standalone simulation with
 * the same parameters, bit for bit. All members must use the same
 * jacobi_iters. */
typedef struct dcg_batch dcg_batch;
typedef struct {
  int32_t tile[4];           /* blocks of 64 cells per CTA (2, 4 or 8) for advect velocity,
                                advect scalars, divergence, apply pressure; 1: one warp per
                                block through shared tiles of the block and its apron      */
  int32_t solve_cache;       /* cells per thread whose stencil the level solve keeps in
                                shared memory: 0, 3, 4 or 8 (8 KB of shared memory each);
                                16 + c (c = 0, 2, 3): pipelined staged sweeps, asynchronous
                                copies into two tile buffers per warp, registers for 3 CTAs
                                per SM, two blocks per claim; 32 + c: three buffers;
                                64 + c (c = 0, 2): two, registers for 5 CTAs per SM;
                                83: two, registers for 4 CTAs per SM, one block per claim */
  int32_t solve_ctas_per_sm; /* CTAs per SM of the cooperative solve (0 = occupancy limit) */
  int32_t solve_barrier;     /* bit 0: grid barrier between sweeps, 0 flat, 1 two-level;
                                bit 1: cascade round r solves every member's level
                                levels-1-r (coarsest levels aligned) instead of level
                                maxtop-r (finest levels aligned); bit 2 (batches of at
                                most 16 members with two level counts): the members of
                                each level count as a separate cascade, the two running
                                concurrently; per-round schedules are then not used      */
  int32_t persistent;        /* cell stages as persistent kernels over the allocated blocks */
  /* per cascade round r < 4: its own schedule when round_ctas_per_sm[r] != 0
   * (CTAs per SM, or -k: one CTA per k SMs; cache depth; barrier), else the
   * solve_* fields above */
  int16_t round_ctas_per_sm[4];
  int8_t round_cache[4];
  int8_t round_barrier[4];
  float solve_ms;            /* autotune: measured time of the whole cascade (all rounds)  */
  float cells_ms[4];         /* autotune: measured time of each cell stage at its tile     */
} dcg_tuning;

int dcg_batch_create(int32_t n, const dcg_params *params, dcg_batch **out);
int dcg_batch_destroy(dcg_batch *batch);
int dcg_batch_reset(dcg_batch *batch);     /* every member as after creation */
int dcg_batch_step(dcg_batch *batch, int32_t n);
/* One batch step without the step graph, timed per stage with CUDA events on
 * the batch's stream (advances the batch like dcg_batch_step(batch, 1)).
 * stage_ms[7]: velocity advection, adaptation, divergence, pressure cascade
 * (with any defect correction), pressure application, scalar advection (each
 * with its fine-to-coarse restriction), the whole step. */
int dcg_batch_profile_step(dcg_batch *batch, float *stage_ms);
int dcg_batch_sync(dcg_batch *batch);      /* stream sync + every member's device error word
                                               (DCG_E_NAN / DCG_E_DEVICE as for dcg_sync) */
/* Borrowed handle of member i for field, stats, topology and emission access
 * (issued on the batch's stream). Stepping, stage calls, set_params,
 * set_stream, set_mode and destroy are refused on member handles. */
int dcg_batch_member(dcg_batch *batch, int32_t i, dcg_sim **out);
int dcg_batch_set_stream(dcg_batch *batch, void *cuda_stream);
/* Autotuner: resets the batch, runs spinup_steps steps, times every candidate
 * tile and solve schedule `reps` times with CUDA events, keeps the fastest,
 * and resets the batch again (the state is that of dcg_batch_reset after it;
 * results do not depend on the tuning). */
int dcg_batch_autotune(dcg_batch *batch, int32_t spinup_steps, int32_t reps, dcg_tuning *out);
int dcg_batch_get_tuning(const dcg_batch *batch, dcg_tuning *out);
int dcg_batch_set_tuning(dcg_batch *batch, const dcg_tuning *tuning);
int dcg_batch_get_info(const dcg_batch *batch, int32_t *n, int64_t *device_bytes, int64_t *launches_per_step);
/* Every member's emission map in one copy (stream-ordered on the batch's
 * stream): maps holds the emission_n^3 maps of the members with emission_n > 0,
 * in member order, consecutively; `where` says whether it is host or device
 * memory. Equivalent to dcg_set_emission on each of those members. */
int dcg_batch_set_emission(dcg_batch *batch, const float *maps, int32_t where);
/* dcg_get_stats of every member (out: n entries), one launch per group of 16
 * members and one synchronisation; DCG_E_NAN (entries filled) when a member's
 * error word holds DCG_DEVERR_NAN */
int dcg_batch_get_stats(dcg_batch *batch, dcg_stats *out);
/* Times the pressure cascade of the current state (all rounds, the members'
 * jacobi_iters sweeps each) `reps` times; *bytes = algorithmic bytes of one
 * cascade, 12 per cell-sweep (p read, div read, p~ write). Leaves p and p~ in
 * an unspecified state until the next step's projection. */
int dcg_batch_time_solve(dcg_batch *batch, int32_t reps, float *avg_ms, double *bytes);
const char *dcg_batch_last_error_string(const dcg_batch *batch);

/* ---- headless renderer (the reference's render(): src/raymarching.cuh,
 * src/dcgrid/dcgrid_rendering.cu, src/uniformgrid/uniformgrid_rendering.cu)
 * ------------------------------------------------------------------------
 * Ray-marches the density into width*height RGBA float4 pixels (row-major,
 * x fastest) in a caller buffer instead of a GL surface. Camera, colours and
 * switches follow the reference's SimParams render fields. */
enum {
  DCG_RENDER_FLUID = 0,      /* density volume, optional sun shadows  */
  DCG_RENDER_DENSITY = 1,    /* debug slice z = gz/2                  */
  DCG_RENDER_VELOCITY = 2,
  DCG_RENDER_FLUIDITY = 3,
  DCG_RENDER_RESOLUTION = 4  /* checker of the sampled cell positions */
};
typedef struct {
  int32_t width, height;
  float eye[3];       /* world units                                       */
  float eye_dir[3];   /* y and z pitch the view about the x axis           */
  float fov;
  float sun_dir[3];   /* unit vector toward the sun                        */
  int32_t aa_samples; /* per axis                                          */
  int32_t channel;    /* DCG_RENDER_*                                      */
  int32_t shadows, solids, precise;
  float ambient;
  float smoke_color[3], scene_color[3], floor_color[3];
  int32_t reserved[4];
} dcg_render_params;
/* the reference's render settings for a width*height image: colours and
 * ambient from SimParams::defaultParams (src/data/sim_params.cpp:16-31);
 * channel, AA samples, solids and shadows as in the frame it displays
 * (src/simulation.cpp:153-156: Fluid, 1, on, on; defaultParams' Resolution
 * channel is overwritten every frame); eye outside the domain looking along +z */
void dcg_default_render_params(dcg_render_params *rp, int32_t width, int32_t height);
int dcg_render(dcg_sim *sim, const dcg_render_params *rp, float *rgba, int32_t where);

/* ---- memory-budget calculator (the reference's scripts/calcMemory*.js,
 * restated for this layout; no GPU needed) ---------------------------------
 * dcg_plan_bytes: device bytes dcg_create(params, mode) allocates (buffers that
 * read-out calls allocate on first use are not included). dcg_blocks_for_budget:
 * the largest max_blocks (params->max_blocks ignored) whose adaptive
 * allocation fits budget_bytes, capped at the full block count of every level
 * (blocks beyond it are never used by any level); DCG_E_BUDGET when not even
 * the coarsest level fits. */
int dcg_plan_bytes(const dcg_params *params, int32_t mode, int64_t *bytes);
int dcg_blocks_for_budget(const dcg_params *params, int64_t budget_bytes, int64_t *max_blocks);

/* ---- state I/O (checkpoint / resume) -------------------------------------
 * No reference counterpart (the reference keeps no on-disk format). The state
 * is everything a step depends on: the block table, neighbour table, level
 * loads and move limits, and the velocity, fluidity, pressure, divergence
 * and scalar fields, after a 64-byte header naming the geometry, budget and
 * storage formats. `where` = DCG_HOST or DCG_DEVICE for the buffer; loading
 * a state into a simulation with a different geometry, budget or format is
 * refused (DCG_E_INVALID). Parameters and the emission map are not part of
 * the state. */
int dcg_state_bytes(dcg_sim *sim, int64_t *bytes);
int dcg_save_state(dcg_sim *sim, void *dst, int32_t where);
int dcg_load_state(dcg_sim *sim, const void *src, int32_t where);

/* ---- adjoint of the density path (extension; no reference counterpart) ------
 * ------------------------------------------------------------------------------
 * With the flow and the topology of the last step held fixed, one step maps
 * the density linearly. dcg_adjoint_step applies the transpose of that map
 * for the step that produced the current state: lam_in (device, 64*max_blocks
 * cells, block-major) is the adjoint of the density after the step;
 * lam_out (device, same size) receives the adjoint of the density before the
 * step; lam_emission (device, emission_n^3, may be NULL) accumulates the
 * adjoint of the emission map. dcg_adjoint_dense adds the transpose of the
 * dense resampling (dcg_get_dense): lam_dense (device, gx*gy*gz) to
 * lam_cells (device, block-major, accumulated). FP32 scalar storage only. */
int dcg_adjoint_step(dcg_sim *sim, const float *lam_in, float *lam_out, float *lam_emission);
int dcg_adjoint_dense(dcg_sim *sim, const float *lam_dense, float *lam_cells);
/* Full adjoint of one step (extension; no reference counterpart): the whole
 * state - velocity and every scalar - with buoyancy, the pressure projection
 * (the transposed cascade: each Jacobi sweep and prolongation transposed, in
 * reverse order) and the dependence of the semi-Lagrangian sample positions
 * on the velocity; the block topology is recorded, not differentiated. The
 * handle must hold the state BEFORE the step: the call runs the step (the
 * handle then holds the state after it, as after dcg_step(sim, 1)) and applies
 * the transposes of its stages in reverse order. lam_in / lam_out: device,
 * (3 + n_scalars) planes of 64*max_blocks cells, block-major: v_x, v_y, v_z,
 * then the scalars; lam_in = the adjoint of the state after the step, lam_out
 * receives that of the state before it (may alias lam_in). lam_emission
 * (device, emission_n^3, may be NULL) accumulates the adjoint of the emission
 * map. FP32 storage, adaptive grid, no defect correction; not for members of
 * a batch. */
int dcg_adjoint_step_full(dcg_sim *sim, const float *lam_in, float *lam_out, float *lam_emission);

/* sizeof of the ABI structs, for binding checks. */
size_t dcg_sizeof_params(void);
size_t dcg_sizeof_info(void);
size_t dcg_sizeof_stats(void);
size_t dcg_sizeof_tuning(void);
size_t dcg_sizeof_render_params(void);

#ifdef __cplusplus
}
#endif
#endif /* DCG_H */
