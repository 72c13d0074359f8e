/*
 * hemelb_gb300.h -- C ABI of the GB300-native lattice-Boltzmann update.
 *
 * This library replaces HemeLB's per-step LB sweep (lb::LBM<Traits>::PreSend /
 * PreReceive / PostReceive over the six collision-type site ranges, with the
 * D3Q19 LBGK/TRT kernels, BulkStreamer, SimpleBounceBack, Bouzidi-Firdaouss-
 * Lallemand, Nash zeroth-order pressure and Ladd velocity link streamers).
 * Every entry point takes plain pointers and sizes; the context owns all device
 * memory; host pointers are borrowed for the duration of the call only.
 *
 * Reference interfaces each entry point stands in for (paths within HemeLB):
 *   hlbg_create            geometry::Domain(latInfo, GmyReadResult, comms) +
 *                          geometry::FieldData(domain) + LBM::Initialise
 *                          (Code/geometry/Domain.cc:26-51, Code/geometry/FieldData.cc:14-25,
 *                           Code/lb/lb.hpp:116-124, InitCollisions :75-114)
 *   hlbg_init_equilibrium  EquilibriumInitialCondition::SetFs (Code/lb/InitialCondition.hpp:40-52)
 *   hlbg_step              one SimulationMaster::DoTimeStep LB part: PreSend + PreReceive +
 *                          PostReceive + FieldData::SwapOldAndNew + SimulationState::Increment
 *                          (Code/lb/lb.hpp:176-309, Code/SimulationMaster.impl.h:218-219)
 *   hlbg_stream_and_collide_range / hlbg_post_step_range
 *                          streamer::StreamAndCollide / PostStep(firstIndex, siteCount, ...)
 *                          (Code/lb/streamers/StreamerTypeFactory.h:48-108, BulkStreamer.h:178-208)
 *   hlbg_swap              FieldData::SwapOldAndNew (Code/geometry/FieldData.h:165-167)
 *   hlbg_get_f / hlbg_put_f FieldData::GetFOld/GetFNew over the contiguous site ids
 *                          (Code/geometry/FieldData.h:117-160)
 *   hlbg_get_macro         MacroscopicPropertyCache density/velocity fill
 *                          (Code/lb/streamers/Common.h:20-42)
 *   hlbg_reduce            StabilityTester::PostSendToParent + ComputeRelativeDifference
 *                          (Code/lb/StabilityTester.h:91-183) plus mass / iolet flux
 *   hlbg_last_error        hemelb::Exception what() (Code/Exception.h)
 */
#ifndef HEMELB_GB300_H
#define HEMELB_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (0 = ok) ------------------------------------------------ */
#define HLBG_OK 0
#define HLBG_ERR_INVAL 1    /* bad argument or inconsistent geometry            */
#define HLBG_ERR_OOM 2      /* device or host allocation failed                 */
#define HLBG_ERR_CUDA 3     /* a CUDA call failed (message in hlbg_last_error)  */
#define HLBG_ERR_UNSTABLE 4 /* a distribution became <= 0 or NaN (StabilityTester) */
#define HLBG_ERR_TIMEOUT 5  /* a bounded device wait gave up                    */
#define HLBG_ERR_STATE 6    /* call not valid in the context's current state    */

/* ---- physics selection (the Traits<> of Code/Traits.h:17-39) --------------- */
#define HLBG_KERNEL_LBGK 0 /* Code/lb/kernels/LBGK.h */
#define HLBG_KERNEL_TRT 1  /* Code/lb/kernels/TRT.h, magic Lambda = 3/16 */

#define HLBG_WALL_SBB 0 /* Code/lb/streamers/SimpleBounceBack.h */
#define HLBG_WALL_BFL 1 /* Code/lb/streamers/BouzidiFirdaousLallemand.h */

#define HLBG_IOLET_NASH 0 /* Code/lb/streamers/NashZerothOrderPressure.h */
#define HLBG_IOLET_LADD 1 /* Code/lb/streamers/LaddIolet.h */

/* storage form of the distributions on the device */
#define HLBG_FP64 0    /* plain form: whole update in FP64                         */
#define HLBG_FP32DEV 1 /* f - w_d stored in FP32, collide in FP32                  */
#define HLBG_FP16 2    /* f - w_d stored in FP16, collide in FP32                  */

/* iolet value models (Code/lb/iolets) */
#define HLBG_IOLET_COSINE 0    /* InOutLetCosine: density(t) = mean + amp cos(2 pi t/T + phase) */
#define HLBG_IOLET_PARABOLIC 1 /* InOutLetParabolicVelocity: n umax (1 - r^2/R^2), warm-up   */
#define HLBG_IOLET_PULSATILE 2 /* parabolic with umax(t) = peak * (1 - cos(2 pi t/T)) / 2    */

/* site types (Code/geometry/SiteType.h) */
#define HLBG_SITE_FLUID 1
#define HLBG_SITE_INLET 2
#define HLBG_SITE_OUTLET 3

/*
 * Sparse block geometry: the content of a GmyReadResult
 * (Code/geometry/GmyReadResult.h) restricted to what the LB update reads.
 * Blocks are 8^3 sites.  A block listed here holds at least one fluid site.
 * Fluid sites whose links are all fluid-fluid need no record; every fluid site
 * with a wall or iolet link has one entry in the link_* arrays.
 * Local site index inside a block: (x * 8 + y) * 8 + z (SiteTraverser order,
 * Code/geometry/VolumeTraverser.cc:22-52).
 */
typedef struct hlbg_geometry {
  int32_t q;                    /* lattice size; 19 (D3Q19); the oracle also takes 15 */
  int32_t block_size;           /* must be 8 */
  int32_t blocks[3];            /* block counts along x, y, z */
  int64_t n_blocks;             /* number of non-empty blocks */
  const int32_t *block_coords;  /* [n_blocks*3] block (i,j,k) */
  const uint64_t *fluid_mask;   /* [n_blocks*8] bit l of word l/64 = site l is fluid */
  int64_t n_link_sites;         /* fluid sites with at least one wall/iolet link */
  const int64_t *link_site;     /* [n] block_index*512 + local site index, ascending */
  const uint32_t *wall_mask;    /* [n] bit d-1 set: link d hits a wall (SiteData) */
  const uint32_t *iolet_mask;   /* [n] bit d-1 set: link d hits an iolet */
  const int32_t *iolet_id;      /* [n] iolet index (into the inlet or outlet list), -1 */
  const int8_t *site_type;      /* [n] HLBG_SITE_* */
  const float *cut_distance;    /* [n*(q-1)] link fraction to the surface, or NULL */
  const float *wall_normal;     /* [n*3] or NULL: wall normal per link site (wall shear stress) */
} hlbg_geometry;

typedef struct hlbg_iolet {
  int32_t model;       /* HLBG_IOLET_COSINE / PARABOLIC / PULSATILE */
  int32_t pad_;
  double position[3];  /* lattice units */
  double normal[3];    /* normalised on create (InOutLet::SetNormal) */
  /* pressure (cosine) iolets */
  double density_mean, density_amp, phase, period;
  /* velocity iolets */
  double radius, max_speed, vel_period;
  uint64_t warmup_steps;
} hlbg_iolet;

typedef struct hlbg_params {
  int32_t kernel;     /* HLBG_KERNEL_* */
  int32_t wall;       /* HLBG_WALL_* */
  int32_t inlet;      /* HLBG_IOLET_NASH / LADD */
  int32_t outlet;     /* HLBG_IOLET_NASH / LADD */
  int32_t precision;  /* HLBG_FP64 / FP32DEV / FP16 */
  int32_t flags;      /* reserved, 0 */
  double tau;         /* relaxation time; omega = -1/tau (LbmParameters::CalcDerivedParams) */
} hlbg_params;

typedef struct hlbg_stats {
  double mass;             /* sum over sites of density (FP64 accumulation) */
  double max_du;           /* max over sites |u_new - u_old| (StabilityTester) */
  double min_f;            /* smallest distribution */
  int64_t unstable_sites;  /* sites with a distribution <= 0 or NaN */
  int64_t time_step;       /* 1-indexed SimulationState time step of the next update */
} hlbg_stats;

/* IncompressibilityChecker's quantities (Code/lb/IncompressibilityChecker.hpp:
 * 157-199) for the state checked by the last monitored step. */
typedef struct hlbg_incomp {
  double min_density;                       /* GetGlobalSmallestDensity */
  double max_density;                       /* GetGlobalLargestDensity */
  double max_velocity;                      /* GetGlobalLargestVelocityMagnitude */
  double max_relative_density_difference;   /* (max - min) / reference density 1 */
  int64_t time_step;                        /* as hlbg_stats; -1 when none */
} hlbg_incomp;

typedef struct hlbg_ctx hlbg_ctx;

/* ---- geometry: synthetic generators (seeded, deterministic) ---------------- */
/* Straight pipe along z, radius R, fluid z in [0, length]; Nash-style inlet at
 * z=-0.5 (normal +z) and outlet at z=length+0.5 (normal -z). */
int hlbg_synth_pipe(double radius, int32_t length, int32_t q, int32_t with_cuts,
                    void **geom_handle);
/* Bifurcation: parent radius/length, daughters by Murray's law (split ratio s in
 * [0.3,0.7]), half-angle in [25,60] degrees, seeded. */
int hlbg_synth_bifurcation(uint64_t seed, double parent_radius, double parent_length,
                           double daughter_length_factor, int32_t q, int32_t with_cuts,
                           void **geom_handle);
/* Stenosed pipe: radius, length, stenosis depth fraction in [0,1). */
int hlbg_synth_stenosis(double radius, int32_t length, double depth, int32_t q,
                        int32_t with_cuts, void **geom_handle);
/* Random vascular forest in a box of box_sites^3 (multiple of 8): n_roots trees
 * of the given depth, root radius, Murray radii, branch angles in [20,70] deg,
 * segment length 6-10 x radius. */
int hlbg_synth_tree(uint64_t seed, int32_t box_sites, int32_t n_roots, int32_t depth,
                    double root_radius, int32_t q, int32_t with_cuts, int32_t n_threads,
                    void **geom_handle);
/* Ensemble of n seeded stenosed pipes (radius 6-20, length 60-240, Gaussian
 * narrowing 0-70%, tau 0.55-1.0) packed into one sparse geometry, one member per
 * cell of blocks with empty blocks between members; inlet m and outlet m belong
 * to member m. */
int hlbg_synth_ensemble(uint64_t seed, int32_t n_members, int32_t q, int32_t n_threads,
                        void **geom_handle);
/* Members of an ensemble: member of each block (in hlbg_geometry block order),
 * per-member tau, shape (radius, length, narrowing) and fluid-site counts (NULL
 * for a single geometry). */
int hlbg_synth_members(void *geom_handle, int32_t *n_members, const int32_t **block_member,
                       const double **member_tau, const double **member_shape,
                       const int64_t **member_sites);
/* Read a HemeLB .gmy geometry file (version 4) for lattice q into a geometry
 * handle (sites re-blocked into 8^3 blocks whatever the file's block size).
 * The file carries no iolet positions: the caller supplies iolets in lattice
 * units.  HLBG_ERR_STATE if the library was built without zlib. */
int hlbg_read_gmy(const char *path, int32_t q, void **geom_handle);
/* Write a sparse block geometry as a HemeLB .gmy file (version 4, 8^3 blocks);
 * lattice links keep type, iolet index and cut distance, other Moore links are
 * NONE, wall sites get the normalised sum of their wall-link vectors as normal. */
int hlbg_write_gmy(const hlbg_geometry *geom, const char *path);
/* Access the generated geometry and its iolets (pointers stay owned by the handle). */
/* One seeded vessel (kind 0: stenosed pipe along z; 1: bifurcation) in a fixed box
 * of box_sites^3 voxels (box_sites a multiple of 8), inlet on the plane z = 1.5
 * and outlets at the far ends, bounce-back walls: the warm-start surrogate's
 * training and held-out geometries.  No reference counterpart. */
int hlbg_synth_vessel_box(uint64_t seed, int32_t box_sites, int32_t kind, int32_t q, void **handle);
/* Signed distance to the wall (positive inside) at every voxel centre of the
 * geometry's box, x slowest and z fastest (box_x * box_y * box_z floats). */
int hlbg_synth_distance(void *handle, float *out);
int hlbg_synth_view(void *geom_handle, hlbg_geometry *out, int64_t *n_fluid_sites,
                    int32_t *n_inlets, int32_t *n_outlets);
int hlbg_synth_iolet(void *geom_handle, int32_t is_outlet, int32_t index, double position[3],
                     double normal[3], double *radius);
void hlbg_synth_free(void *geom_handle);

/* ---- solver context -------------------------------------------------------- */
int hlbg_create(const hlbg_geometry *geom, const hlbg_params *params,
                const hlbg_iolet *inlets, int32_t n_inlets, const hlbg_iolet *outlets,
                int32_t n_outlets, hlbg_ctx **out);
/* Replace the iolets' parameters (BoundaryValues' iolets,
 * Code/lb/iolets/BoundaryValues.h:21,83): same counts as at creation (the
 * geometry's iolet ids refer to them), models matching the streamers; the next
 * step uses the new densities / velocities, positions and normals. */
int hlbg_set_iolets(hlbg_ctx *ctx, const hlbg_iolet *inlets, int32_t n_inlets,
                    const hlbg_iolet *outlets, int32_t n_outlets);
void hlbg_destroy(hlbg_ctx *ctx);
const char *hlbg_last_error(const hlbg_ctx *ctx);

int64_t hlbg_site_count(const hlbg_ctx *ctx);   /* fluid sites N */
int64_t hlbg_slot_count(const hlbg_ctx *ctx);   /* device slots (n_blocks * 512) */
/* Kernel launches one hlbg_step time step makes (stream-collide, iolet links, BFL PostStep). */
int32_t hlbg_launches_per_step(const hlbg_ctx *ctx);
int hlbg_collision_counts(const hlbg_ctx *ctx, int64_t counts[6]);
size_t hlbg_device_bytes(const hlbg_ctx *ctx);

/* Permutation: ref_to_slot[i] = device slot of contiguous site id i (ref order:
 * collision type, then Morton block order, then in-block order). */
int hlbg_site_order(const hlbg_ctx *ctx, int64_t *ref_to_slot);

/* Global coordinates of the sites in contiguous order (xyz[N*3]; Domain::GetGlobalSiteCoords). */
int hlbg_site_coords(const hlbg_ctx *ctx, int32_t *xyz);

/* Uniform equilibrium initial condition (both f arrays), time step reset to 1. */
int hlbg_init_equilibrium(hlbg_ctx *ctx, double density, double vx, double vy, double vz);
/* Per-site equilibrium start from host fields in contiguous site order
 * (rho[N], u[N*3]); the learned warm-start hook. */
int hlbg_init_equilibrium_field(hlbg_ctx *ctx, const double *rho, const double *u);

/* Advance nsteps full time steps on the given CUDA stream (NULL = context stream).
 * Returns after enqueueing; hlbg_sync waits. */
int hlbg_step(hlbg_ctx *ctx, int32_t nsteps, void *cuda_stream);
int hlbg_sync(hlbg_ctx *ctx);
/* Same as hlbg_step, as CUDA graph launches: every kernel of up to 1024 steps is
 * captured once per step count and replayed (launch-bound small geometries and
 * batched ensembles). */
int hlbg_step_graph(hlbg_ctx *ctx, int32_t nsteps);
/* Step until the state is steady: StabilityTester's convergence test, max over
 * sites of |u_new - u_old| / u_ref <= tol, checked on the device after every step
 * (Code/lb/StabilityTester.h:91-183 with doConvergenceCheck, and the termination
 * on convergence of SimulationMaster).  Steps run as graph launches of check_batch
 * (1..1024) steps; the host reads the result after each, so steps_run exceeds
 * steps_to_steady by less than check_batch.  Returns HLBG_OK when converged,
 * HLBG_ERR_UNSTABLE when a distribution turned non-positive, HLBG_ERR_TIMEOUT
 * after max_steps; final_rel_du is the last check's max |du| / u_ref. */
int hlbg_run_to_steady(hlbg_ctx *ctx, double tol, double u_ref, int64_t max_steps,
                       int32_t check_batch, int64_t *steps_to_steady, int64_t *steps_run,
                       double *final_rel_du);
/* nsteps time steps with the StabilityTester fused into the update (each site's
 * velocity is recorded as it collides; the change against the previous record,
 * f > 0 and the mass are reduced on the device).  The check of step k is made while
 * step k + 1 collides, so the stats returned are those of the step before the last
 * one (time_step = that step + 1, SimulationState's count when the reference makes
 * the check), or time_step = -1 when there is none yet: the first step after the
 * distributions were set or changed outside a monitored step only records.
 * Replaces hlbg_step + hlbg_reduce per step without re-reading both arrays
 * (Code/lb/StabilityTester.h:91-183).
 * With a check interval K > 1 (hlbg_set_monitor_interval) only the steps t with
 * t % K == 0 check; the step before each records the velocities and the others run
 * the plain update, so the stats are those of the last check (time_step = its t,
 * or -1 when none was made).  The reference checks on the cycle of its phased
 * broadcast: every step on one rank, every 2 * tree-depth steps on many ranks
 * (net::PhasedBroadcastRegular, Code/net/PhasedBroadcastRegular.h:106-182).
 * K = 1 (the default) checks every step as described above. */
int hlbg_step_monitored(hlbg_ctx *ctx, int32_t nsteps, hlbg_stats *out);
int hlbg_set_monitor_interval(hlbg_ctx *ctx, int32_t interval);
/* Mass flux through each iolet of the current state: out[k] (inlets first, then
 * outlets; n = their total) sums, over the sites with links to that iolet, the
 * site's momentum sum_d c_d f_d along the iolet's normalised inward normal, in
 * FP64, in a fixed order.  Inflow is positive at inlets and negative at outlets;
 * at steady state the sum over all iolets is ~0.  No reference counterpart (the
 * per-iolet flux of the monitoring reductions). */
int hlbg_iolet_flux(hlbg_ctx *ctx, double *out, int32_t n);
/* XTR distribution checkpoints (doc/dev/file-formats/extraction.md, version 5): one
 * field "distributions" of 19 doubles per site, sites in contiguous order with their
 * grid positions, one record per timestep, and the ".off" offset file of a single
 * rank, as LocalPropertyOutput writes them (Code/extraction/LocalPropertyOutput.cc)
 * and LocalDistributionInput reads them (LocalDistributionInput.cc:56-251).
 * hlbg_write_checkpoint writes the current state (the reference's fOld) at
 * `timestep`; with append != 0 it adds a record to an existing file of the same
 * geometry, and refuses (HLBG_ERR_INVAL, file unchanged) a timestep that is not
 * larger than the file's last, since the reader finds a timestep by binary search
 * over records in increasing order.  hlbg_read_checkpoint loads the record of `timestep` (the last one when
 * timestep < 0) into both time levels after checking every site's position, and
 * reports the timestep it found. */
int hlbg_write_checkpoint(hlbg_ctx *ctx, const char *path, uint64_t timestep, double voxel_size,
                          const double origin[3], int32_t append);
int hlbg_read_checkpoint(hlbg_ctx *ctx, const char *path, int64_t timestep, uint64_t *found);
/* Wall shear stress magnitude of every site of the current state, in contiguous
 * site order (out[N]): Lattice::CalculateWallShearStressMagnitude on f_neq with the
 * site's wall normal and LbmParameters' stress parameter (1 - 1/(2 tau)) / sqrt(2),
 * as UpdateCachePostCollision fills wallShearStressMagnitudeCache
 * (Code/lb/streamers/Common.h:35-52); DBL_MAX (NO_VALUE) where the site has no wall
 * link.  Normals are the geometry's wall_normal, else the normalised sum of the
 * site's wall-link vectors.  Computed in FP64 for every storage form. */
int hlbg_wall_shear_stress(hlbg_ctx *ctx, double *out);
/* IncompressibilityChecker for the state checked by the last monitored step
 * (hlbg_step_monitored or hlbg_run_to_steady): the densities and velocities are
 * those of the state each site collided, as the reference's property cache holds
 * them after a step.  IsDensityDiffWithinRange is
 * max_relative_density_difference < 0.05 with the reference's default. */
int hlbg_incompressibility(hlbg_ctx *ctx, hlbg_incomp *out);
/* Replace the current distributions by the mean of the two time levels (valid
 * right after a step, when both arrays hold consecutive states).  No reference
 * counterpart: applied once after the first step of a start from a prescribed
 * field, it removes the period-two staggered-momentum component that D3Q19 with
 * bounce-back walls conserves everywhere except at iolets (sum over sites of
 * (-1)^(z+t) j_z, and likewise for x and y), which otherwise decays only through
 * the iolets and dominates the time to steady state. */
int hlbg_average_time_levels(hlbg_ctx *ctx);
/* Select the stream-and-collide launch shape by index (0..8: all slots at 128x10,
 * 128x8, 256x4, 512x2 threads x resident CTAs; one CTA per block with the block's
 * fluid rows staged in shared memory by bulk asynchronous copies (FP32 / FP16;
 * FP64 runs index 6 instead); the fluid list, whose warps hold only fluid slots,
 * at 128x9, 128x8 and 64x16; one persistent CTA per SM whose producer warp stages
 * blocks into a ring of shared-memory buffers by bulk asynchronous copies ahead of
 * 31 consumer warps (FP32 / FP16; FP64 runs index 6 instead)); FP64 runs two
 * CTAs per SM.  Monitored steps run every index from 4 up as the 128x8 fluid
 * list.  No reference counterpart. */
int hlbg_set_launch_variant(hlbg_ctx *ctx, int32_t variant);
/* Autotuner: time each launch shape / schedule of the stream-and-collide kernel
 * (threads per CTA x resident CTAs per SM, per-slot grid or persistent grid) on
 * this context for steps_per_trial steps and keep the fastest.  Advances the
 * state like hlbg_step.  chosen / best_ms may be NULL. */
int hlbg_autotune(hlbg_ctx *ctx, int32_t steps_per_trial, int32_t *chosen, float *best_ms);
/* Per-block relaxation time (input block order), e.g. one tau per ensemble member;
 * omega = -1/tau per block (LbmParameters::CalcDerivedParams). */
int hlbg_set_block_tau(hlbg_ctx *ctx, const double *tau_per_block);

/* Per-range drop-in for one streamer: ranges are contiguous site ids. */
int hlbg_stream_and_collide_range(hlbg_ctx *ctx, int64_t first, int64_t count);
int hlbg_post_step_range(hlbg_ctx *ctx, int64_t first, int64_t count);
int hlbg_swap(hlbg_ctx *ctx); /* SwapOldAndNew + time step increment */
/* Set the 1-indexed time step of the next update (SimulationState::GetTimeStep;
 * Code/lb/SimulationState.cc:40-48), e.g. after loading a checkpoint. */
int hlbg_set_time_step(hlbg_ctx *ctx, uint64_t t1);

/* Distributions in contiguous site order, AoS [N*q] doubles (FieldData layout).
 * which = 0: fOld (current), 1: fNew. */
int hlbg_get_f(hlbg_ctx *ctx, double *host, int32_t which);
int hlbg_put_f(hlbg_ctx *ctx, const double *host, int32_t which);
/* Same, device pointers (stream-ordered on the context stream). */
int hlbg_get_f_device(hlbg_ctx *ctx, double *dev, int32_t which);
int hlbg_put_f_device(hlbg_ctx *ctx, const double *dev, int32_t which);

/* Density and velocity per site (contiguous order) from the current f. */
int hlbg_get_macro(hlbg_ctx *ctx, double *rho, double *u);

/* StabilityTester reductions over the two time levels the context holds: mass
 * and min f of the current distributions, unstable-site count (f <= 0 or not
 * finite), and max|du| between the velocity of the current and of the previous
 * time level (the last step's input), so a call depends on no earlier call.
 * Synchronous.  Allocates its partial-sum buffer on its first call. */
int hlbg_reduce(hlbg_ctx *ctx, hlbg_stats *out);

/* Allocation-free variant of hlbg_reduce.  No counterpart in the reference: it
 * exists for callers that must not allocate device memory once their time loop
 * runs -- a host framework that reserves its whole device-memory budget up front,
 * or one for which a cudaMalloc in the loop would synchronise the device and stall
 * overlapped work -- whereas hlbg_reduce allocates its partial-sum buffer on its
 * first call.  Scratch is a fixed 2 MiB static device array (one partial per
 * 256-slot reduction block), so geometries are limited to HLBG_NOALLOC_MAX_SLOTS
 * slots (hlbg_slot_count); larger ones are rejected with HLBG_ERR_INVAL.
 * The array is placed on a GPU when the library's device code first loads there:
 * at library load, or -- with lazy module loading, CUDA's default -- during the
 * first hlbg_create on that device, which also looks up the array's device
 * address (with the device current) and loads the reduction kernels, so no call
 * of this function loads or allocates anything.  Every GPU that has held a
 * context keeps the 2 MiB until the process exits.  A context does not survive a
 * reset of its device (cudaDeviceReset); contexts created afterwards look the
 * array up again.  All calls on a device share the array: calls that overlap on
 * the GPU race.  Synchronous, same results as hlbg_reduce. */
#define HLBG_NOALLOC_MAX_SLOTS (65536LL * 256LL)
int hlbg_reduce_noalloc(hlbg_ctx *ctx, hlbg_stats *out);

/* Per-step iolet values the host computed for the steps [t, t+n) (for tests). */
int hlbg_iolet_density(const hlbg_ctx *ctx, int32_t is_outlet, int32_t index, uint64_t t,
                       double *density);

/* Measurement helper: enqueue nsteps with hlbg_step and return the elapsed time
 * between CUDA events recorded on the context stream around them (ms). */
int hlbg_time_steps(hlbg_ctx *ctx, int32_t nsteps, float *ms);
/* Same as hlbg_step(nsteps) with events around every launch: summed device time
 * of the stream-and-collide launches and of the BFL PostStep launches (ms). */
int hlbg_time_kernels(hlbg_ctx *ctx, int32_t nsteps, float *collide_ms, float *post_ms);

/* ---- multi-rank halo: host-side index maps --------------------------------
 * Splits one geometry over ranks for a device update per rank with one exchange
 * per step, in place of the reference's domain decomposition and
 * geometry::FieldData::SendAndReceive / CopyReceived (Code/geometry/FieldData.cc:
 * 27-49) with lb::LBM's edge-first / mid-second order (Code/lb/lb.hpp:176-309).
 * Host work only: no device memory, no CUDA call.
 *
 * hlbg_halo_partition: rank of every input block (block_rank[n_blocks]):
 *   contiguous ranges of the device block order (z-columns: 2-D Morton order of
 *   the block's (x, y), then z) cut where the running fluid-site count passes
 *   k*N/n_ranks.  Any other assignment may be passed to hlbg_halo_create.
 * hlbg_halo_create: the index maps of `rank`.  Its local geometry holds the owned
 *   blocks, then every block of another rank that neighbours an owned block
 *   (ghost blocks), with their link records, so an owned site sees the same
 *   neighbourhood as in the whole geometry; a context created on it updates the
 *   owned sites exactly as the whole geometry's context would once the received
 *   distributions are in place.  Per peer, two lists of (local block, direction,
 *   in-block site) triples: send = the distributions this rank's owned sites
 *   stream into the peer's sites (found in this rank's new distributions at the
 *   ghost sites), receive = those the peer streams into this rank's sites.  A
 *   send list and the peer's receive list name the same distributions in the same
 *   order (ascending target block, site, direction of the input geometry).
 *   Exchange after StreamAndCollide, before PostStep.  D3Q19 only.
 * hlbg_halo_edge_blocks: per owned block, 1 when one of its sites streams into a
 *   ghost block (update these first and send; update the others meanwhile).
 * hlbg_halo_block_source: input block index of every local block.
 * The halo owns the arrays of its local geometry view; the view is valid until
 * hlbg_halo_destroy.  Errors: HLBG_ERR_INVAL with hlbg_halo_last_error. */
typedef struct hlbg_halo hlbg_halo;
int hlbg_halo_partition(const hlbg_geometry *g, int32_t n_ranks, int32_t *block_rank);
int hlbg_halo_create(const hlbg_geometry *g, const int32_t *block_rank, int32_t n_ranks, int32_t rank,
                     hlbg_halo **out);
void hlbg_halo_destroy(hlbg_halo *h);
const char *hlbg_halo_last_error(const hlbg_halo *h);
int hlbg_halo_local_geometry(const hlbg_halo *h, hlbg_geometry *out, int64_t *n_owned_blocks);
int hlbg_halo_block_source(const hlbg_halo *h, int64_t *input_block);
int hlbg_halo_edge_blocks(const hlbg_halo *h, uint8_t *is_edge);
int32_t hlbg_halo_peer_count(const hlbg_halo *h);
int hlbg_halo_peer(const hlbg_halo *h, int32_t k, int32_t *peer_rank, int64_t *n_send, int64_t *n_recv);
int hlbg_halo_list(const hlbg_halo *h, int32_t k, int32_t is_recv, int32_t *local_block, int8_t *direction,
                   int16_t *site);

/* Device half of the exchange, for a context created on a halo's local geometry.
 * hlbg_halo_offsets: element offsets, in the context's distribution arrays, of
 *   (block, direction, in-block site) triples, block indexing the geometry given
 *   to hlbg_create (for a halo's lists: its local blocks).  Host work.
 * hlbg_halo_pack_device / hlbg_halo_unpack_device: copy the new distributions
 *   (the state StreamAndCollide wrote, before PostStep and the swap) at device
 *   `offsets` into / from a device buffer of n elements of the storage type
 *   (hlbg_storage_bytes: 8 FP64, 4 FP32-deviation, 2 FP16), so the exchange is
 *   exact in every form.  Enqueued on the context stream; offsets outside the
 *   arrays are skipped and reported by the next hlbg_halo_check (which
 *   synchronises the stream). */
int hlbg_halo_offsets(hlbg_ctx *ctx, const int32_t *block, const int8_t *direction, const int16_t *site,
                      int64_t n, int64_t *out);
int hlbg_halo_pack_device(hlbg_ctx *ctx, const int64_t *offsets, int64_t n, void *buf);
int hlbg_halo_unpack_device(hlbg_ctx *ctx, const int64_t *offsets, int64_t n, const void *buf);
int hlbg_halo_check(hlbg_ctx *ctx);
int hlbg_storage_bytes(const hlbg_ctx *ctx);

/* Library build string. */
const char *hlbg_version(void);

#ifdef __cplusplus
}
#endif
#endif /* HEMELB_GB300_H */
