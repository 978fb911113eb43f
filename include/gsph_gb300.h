/*
 * gsph_gb300.h — C ABI of the GB300 grad-h SPH + KD-tree gravity particle step.
 *
 * One context holds one simulation's particles on one GPU.  The entry points replace the
 * virtual methods a GANDALF Simulation calls on its SphNeighbourSearch object
 * (GradhSphTree<ndim,GradhSphParticle>, src/Headers/SphNeighbourSearch.h:173-227):
 *
 *   gsph_build_tree                   <- HydroTree::BuildTree            src/Tree/HydroTree.cpp:309-372
 *                                        (rebuild branch; also replaces BuildGhostTree
 *                                        :381-441 and SearchBoundaryGhostParticles :494-543,
 *                                        whose periodic images the kernels form on the fly)
 *   gsph_update_all_sph_properties    <- GradhSphTree::UpdateAllSphProperties
 *                                                                        src/GradhSph/GradhSphTree.cpp:82-271
 *   gsph_update_all_sph_hydro_forces  <- GradhSphTree::UpdateAllSphHydroForces  :279-435
 *   gsph_update_all_sph_forces        <- GradhSphTree::UpdateAllSphForces       :443-657
 *   gsph_update_all_star_gas_forces   <- HydroTree::UpdateAllStarGasForces src/Tree/HydroTree.cpp:551-654
 *
 * Particles cross the boundary either as structure-of-arrays (plain double pointers) or
 * as the caller's array-of-structures (GradhSphParticle records, Particle.h:285-368)
 * described by byte offsets.  All calls are synchronous with respect to the host unless
 * stated; none allocate pinned host memory; none abort the process.
 *
 * Return codes: GSPH_OK (0), a negative GSPH_ERR_* code on failure.  The context keeps
 * a message for the last failure (gsph_last_error).
 */
#ifndef GSPH_GB300_H_
#define GSPH_GB300_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GSPH_ABI_VERSION 3

#define GSPH_OK 0
#define GSPH_ERR_INVALID -1        /* bad argument or particle data */
#define GSPH_ERR_CUDA -2           /* CUDA runtime failure */
#define GSPH_ERR_UNSUPPORTED -3    /* option outside the implemented path */
#define GSPH_ERR_STATE -4          /* call made out of order (e.g. forces before h solve) */
#define GSPH_ERR_NOT_CONVERGED -5  /* h-rho iteration failed; the reference raises
                                      "Problem with convergence of h-rho iteration" */
#define GSPH_ERR_CAPACITY -6       /* walk stack or hmax retry limit exhausted */

typedef struct gsph_ctx gsph_ctx;

enum gsph_eos { GSPH_EOS_ENERGY_EQN = 0, GSPH_EOS_ISOTHERMAL = 1 };
enum gsph_multipole { GSPH_MONOPOLE = 0, GSPH_QUADRUPOLE = 1 };
enum gsph_precision { GSPH_PRECISION_FP64 = 0, GSPH_PRECISION_MIXED = 1 };

/* Run parameters; names follow the GANDALF parameter keys (src/Common/Parameters.cpp). */
typedef struct gsph_config {
  int32_t ndim;          /* must be 3 */
  int32_t nleafmax;      /* "Nleafmax" (KD-tree leaf size), 1..32 */
  int32_t hydro_forces;  /* "hydro_forces" */
  int32_t self_gravity;  /* "self_gravity" */
  int32_t eos;           /* "gas_eos": energy_eqn or isothermal */
  int32_t multipole;     /* "multipole": monopole or quadrupole (geometric MAC) */
  int32_t periodic;      /* 1: periodic in x, y and z ("boundary_lhs/rhs" = periodic) */
  int32_t precision;     /* GSPH_PRECISION_FP64 or GSPH_PRECISION_MIXED (at most 2^27
                            particles: larger sets return GSPH_ERR_UNSUPPORTED) */
  double h_fac;          /* "h_fac" */
  double h_converge;     /* "h_converge" */
  double alpha_visc;     /* "alpha_visc" (avisc = mon97) */
  double beta_visc;      /* "beta_visc" */
  double gamma_eos;      /* "gamma_eos" */
  double temp0;          /* "temp0" (isothermal) */
  double mu_bar;         /* "mu_bar" (isothermal) */
  double thetamaxsqd;    /* "thetamaxsqd" (geometric opening angle squared) */
  double boxmin[3];      /* "boxmin[k]" (periodic box) */
  double boxmax[3];      /* "boxmax[k]" */
  int32_t compensated;   /* mixed form: 1 = compensated (Kahan) float sums for the density and
                            gravity accumulations, the lanes' partials combined in FP64 */
  int32_t reserved;      /* must be 0 */
} gsph_config;

/* Byte offsets of the fields inside one array-of-structures particle record
 * (GradhSphParticle<3>, src/Headers/Particle.h:133-368).  r, v, a and atree point at 3
 * consecutive doubles; flags, level and levelneib at 32-bit integers.  An offset of -1
 * skips that field.
 *
 * Without flags (flags = -1) every particle is active: the calls solve and write every
 * particle.  With flags, the reference's block-timestep semantics hold: a particle is
 * active when its flags have the `active` bit (1 << 1, src/Headers/Flags.h:33); the h
 * solve and the force passes compute active particles only (GradhSphTree.cpp:96-102,
 * :300-305), the other particles keep the solved state their records hold at import
 * (rho, invomega, zeta, hfactor, hrangesqd, pressure, sound, a, atree, gpot, dudt, div_v,
 * gpot_hydro are then read as well), and levelneib is maintained as the reference does
 * (GradhSphTree.cpp:375-417, :619-640). */
typedef struct gsph_field_offsets {
  int64_t r, v, m, h, u;                                   /* inputs */
  int64_t rho, invomega, zeta, hfactor, hrangesqd, pressure, sound, div_v, dudt, a, atree,
      gpot, gpot_hydro;                                    /* outputs */
  int64_t flags, level, levelneib;                         /* block timesteps (int32 fields) */
} gsph_field_offsets;

#define GSPH_FLAG_ACTIVE 2u    /* the reference's `active` particle flag */

/* Per-particle output fields for gsph_get_field (input order). */
enum gsph_field {
  GSPH_FIELD_H = 0, GSPH_FIELD_RHO, GSPH_FIELD_INVOMEGA, GSPH_FIELD_ZETA, GSPH_FIELD_HFACTOR,
  GSPH_FIELD_PRESSURE, GSPH_FIELD_SOUND, GSPH_FIELD_U, GSPH_FIELD_DIV_V, GSPH_FIELD_DUDT,
  GSPH_FIELD_AX, GSPH_FIELD_AY, GSPH_FIELD_AZ, GSPH_FIELD_AGX, GSPH_FIELD_AGY, GSPH_FIELD_AGZ,
  GSPH_FIELD_GPOT, GSPH_FIELD_HRANGESQD, GSPH_FIELD_GPOT_HYDRO, GSPH_FIELD_COUNT
};

/* Counters of the last step: interactions evaluated (used for the roofline), the
 * status word of the kernels and the device time of each phase in milliseconds. */
typedef struct gsph_stats {
  int64_t n, ncell, nleaf, ltot;
  int64_t density_pairs;   /* pair evaluations inside the kernel support, all iterations */
  int64_t hydro_pairs;     /* SPH pairs of the force pass */
  int64_t direct_pairs;    /* Newtonian particle-particle terms */
  int64_t cell_pairs;      /* particle-multipole terms */
  int64_t exact_checks;    /* mixed form: membership tests re-resolved in fp64 */
  int64_t heavy_density;   /* leaf cells the h solve handed to its wide kernel */
  int64_t heavy_forces;    /* leaf cells the force pass handed to its wide kernel */
  uint32_t status;
  uint32_t launches;       /* kernels this library launched for the last step */
  double ms_build, ms_density, ms_hmax, ms_forces, ms_total;
} gsph_stats;

/* ---- lifetime ------------------------------------------------------------------------- */
int32_t gsph_abi_version(void);
void gsph_config_defaults(gsph_config* cfg);     /* GANDALF defaults, kernel m4, Nleafmax 8 */
gsph_ctx* gsph_create(const gsph_config* cfg, int32_t device);   /* NULL on failure */
void gsph_destroy(gsph_ctx* ctx);
const char* gsph_last_error(const gsph_ctx* ctx);
int32_t gsph_create_error(void);                  /* code of the last failed gsph_create */

/* Launch all further work of this context on the caller's CUDA stream (a cudaStream_t;
 * NULL restores the context's own stream).  Calls still synchronise that stream before
 * returning results to the host. */
int32_t gsph_set_stream(gsph_ctx* ctx, void* stream);

/* Measured fused multiply-add throughput of this GPU in GFLOP/s (2 flops per FMA):
 * fp64 = 1 for double, 0 for float.  A calibration aid for roofline fractions of the
 * pair loops, which run on the FP64 / FP32 pipes rather than tensor cores. */
double gsph_fma_peak_gflops(int32_t device, int32_t fp64);

/* ---- particle import (Simulation::ImportArraySph, src/Common/Simulation.cpp:1442) ------ */
/* Host structure-of-arrays, n particles, input order.  Copies into device memory. */
int32_t gsph_set_particles(gsph_ctx* ctx, int64_t n, const double* x, const double* y,
                           const double* z, const double* vx, const double* vy, const double* vz,
                           const double* m, const double* u, const double* h);
/* Same, from device pointers (no host traffic). */
int32_t gsph_set_particles_device(gsph_ctx* ctx, int64_t n, const double* x, const double* y,
                                  const double* z, const double* vx, const double* vy,
                                  const double* vz, const double* m, const double* u,
                                  const double* h);
/* Host array-of-structures (the reference's GradhSphParticle array): record stride and
 * field offsets in bytes.  The input fields (and, with flags, the flags, levels and solved
 * state above) are read from the records; nothing else of a record is read or kept.
 * Records in page-locked memory (cudaHostAlloc / cudaHostRegister) are read in place by a
 * kernel; other records are copied to the device whole and unpacked there. */
int32_t gsph_set_particles_aos(gsph_ctx* ctx, const void* base, int64_t n, int64_t stride,
                               const gsph_field_offsets* off);
/* KDTree::UpdateActiveParticleCounters (src/Tree/KDTree.cpp:1217; called by MainLoop before
 * a repeated pass, src/Hydrodynamics/SphSimulation.cpp:643): re-read the flags and levels
 * of the records (after CheckTimesteps changed them) into the current tree, without a
 * rebuild.  The records and offsets are those of gsph_set_particles_aos, with flags. */
int32_t gsph_update_active_particle_counters(gsph_ctx* ctx, const void* base, int64_t n, int64_t stride,
                                             const gsph_field_offsets* off);
/* HydroTree::GetMaximumSmoothingLength (src/Tree/HydroTree.cpp:661): the largest h in the
 * tree (root cell hmax) after the last tree build or h solve. */
int32_t gsph_get_maximum_smoothing_length(gsph_ctx* ctx, double* hmax);

/* ---- star particles (Simulation::ImportArrayNbody, src/Common/Simulation.cpp:1325-1430;
 *      the stars a Simulation keeps in Nbody::nbodydata) ---------------------------------- */
/* Host structure-of-arrays of nstar stars: position, velocity, mass, softening length h.
 * nstar = 0 removes them.  With stars set, the h solve adds the SPH-star zeta term
 * (GradhSph::ComputeH, src/GradhSph/GradhSph.cpp:282-297), both gas force passes add the
 * stars' softened gravity to a, atree and gpot after gpot_hydro is taken
 * (GradhSph::ComputeStarGravForces, src/GradhSph/GradhSph.cpp:698-743), and gsph_step
 * with self-gravity also computes the star <- gas forces.  Setting stars invalidates the
 * solved smoothing lengths and forces. */
int32_t gsph_set_stars(gsph_ctx* ctx, int64_t nstar, const double* x, const double* y, const double* z,
                       const double* vx, const double* vy, const double* vz, const double* m,
                       const double* h);
/* Gravity of the gas on every star through the gas tree (a, adot and gpot of the gas
 * alone; the caller adds star-star terms).  Needs self-gravity and a solved h. */
int32_t gsph_update_all_star_gas_forces(gsph_ctx* ctx);
/* The star <- gas results into host arrays of nstar doubles (any pointer may be NULL). */
int32_t gsph_get_star_forces(gsph_ctx* ctx, double* ax, double* ay, double* az, double* adotx,
                             double* adoty, double* adotz, double* gpot);

/* ---- the step ---------------------------------------------------------------------------- */
int32_t gsph_build_tree(gsph_ctx* ctx);
int32_t gsph_update_all_sph_properties(gsph_ctx* ctx);   /* h-rho solve + tree hmax update */
int32_t gsph_update_all_sph_hydro_forces(gsph_ctx* ctx);
int32_t gsph_update_all_sph_forces(gsph_ctx* ctx);        /* hydro + self-gravity */
/* build + properties + forces (hydro only or hydro + gravity, as configured) */
int32_t gsph_step(gsph_ctx* ctx);
/* The same step replayed from a CUDA graph: the step's launches are captured once and
 * re-captured automatically when the particle count, the stars or the recording setting
 * change (the particle values may change freely between calls).  Results are identical
 * to gsph_step's. */
int32_t gsph_step_graph(gsph_ctx* ctx);

/* ---- KDK leapfrog with block timesteps --------------------------------------------------
 * The gas part of SphSimulation::PostInitialConditionsSetup and MainLoop
 * (src/Hydrodynamics/SphSimulation.cpp:203-565, :573-880) with SphLeapfrogKDK
 * (src/Hydrodynamics/SphLeapfrogKDK.cpp) and Simulation::ComputeBlockTimesteps
 * (src/Common/Simulation.cpp:1764-2190), run on the device: every step drifts all
 * particles, rebuilds the tree, solves h and the forces of the active particles (those at
 * the end of their step), repeats for particles the neighbour-timestep check activates,
 * assigns new timestep levels and closes the steps that end.  The integer-time state stays
 * on the device, so a sequence of steps needs no host round trip and can run as one CUDA
 * graph.  Parameters as the reference's Nlevels, level_diff_max, courant_mult, accel_mult,
 * energy_mult (Parameters.cpp:239-263); the energy equation is integrated for gas_eos =
 * energy_eqn.  Stars are not supported here. */
typedef struct gsph_kdk_config {
  int32_t nlevels, level_diff_max;
  double courant_mult, accel_mult, energy_mult;
} gsph_kdk_config;
void gsph_kdk_config_defaults(gsph_kdk_config* cfg);
/* Initial h solves, forces and timesteps for the imported particles (time 0). */
int32_t gsph_kdk_setup(gsph_ctx* ctx, const gsph_kdk_config* cfg);
/* nsteps main-loop steps; use_graph = 1 replays them from one captured CUDA graph. */
int32_t gsph_kdk_steps(gsph_ctx* ctx, int32_t nsteps, int32_t use_graph);
typedef struct gsph_kdk_status {
  int64_t n, nresync, level_max, level_step, nsteps;   /* integer time (Simulation.h:187-215) */
  double t, timestep, dt_max;
  int64_t active_updates;     /* active particles summed over all force passes since setup */
  uint32_t status;            /* 1: invalid timestep, 2: timestep checks did not settle */
} gsph_kdk_status;
int32_t gsph_kdk_get_status(gsph_ctx* ctx, gsph_kdk_status* out);
/* Device time and interaction counts of the last gsph_kdk_steps call, for roofline
 * accounting: tree builds, and the first h solve and force pass of every step (timed with
 * CUDA events on the context's stream); the CheckTimesteps repeat passes run as conditional
 * graph nodes, which hold no events, and are counted in repeat_passes only (the repeat
 * passes found no active particle are skipped altogether). */
typedef struct gsph_kdk_timing {
  double ms_build, ms_density, ms_forces;
  int64_t density_pairs, hydro_pairs, direct_pairs, cell_pairs;   /* of the first passes */
  int64_t steps, repeat_passes;
} gsph_kdk_timing;
int32_t gsph_kdk_get_timing(gsph_ctx* ctx, gsph_kdk_timing* out);
enum gsph_kdk_field {
  GSPH_KDK_X = 0, GSPH_KDK_Y, GSPH_KDK_Z, GSPH_KDK_VX, GSPH_KDK_VY, GSPH_KDK_VZ, GSPH_KDK_U, GSPH_KDK_DT,
  GSPH_KDK_TLAST, GSPH_KDK_LEVEL, GSPH_KDK_NSTEP, GSPH_KDK_NLAST, GSPH_KDK_LEVELNEIB, GSPH_KDK_COUNT
};
/* One integration field for all particles, input order, as doubles (n values). */
int32_t gsph_kdk_get_state(gsph_ctx* ctx, int32_t which, double* out);

/* ---- batches of independent simulations ------------------------------------------------
 * No counterpart in the reference (which steps one simulation per process).  A batch
 * steps many mixed-precision contexts at once: each of the density and force passes is one
 * persistent launch whose warps pull leaf cells of all simulations from a device work
 * queue, and the per-simulation tree builds and cell updates run as parallel branches of
 * one CUDA graph.  Results per context are identical to gsph_step on that context; read
 * them with the per-context calls.  All contexts must be mixed precision on one device,
 * share the self_gravity setting and have no stars; a context may belong to one batch at a
 * time and must not be stepped on its own while the batch step runs. */
typedef struct gsph_batch gsph_batch;
gsph_batch* gsph_batch_create(gsph_ctx* const* ctxs, int32_t nsim);   /* NULL: see gsph_create_error */
void gsph_batch_destroy(gsph_batch* batch);
int32_t gsph_batch_step(gsph_batch* batch);
const char* gsph_batch_last_error(const gsph_batch* batch);
/* Device time of the last batch step (ms) and the kernels one batch step launches. */
int32_t gsph_batch_stats(const gsph_batch* batch, float* ms, int32_t* launches);

/* ---- results ----------------------------------------------------------------------------- */
/* One field for all particles in input order into host memory (n doubles). */
int32_t gsph_get_field(gsph_ctx* ctx, int32_t field, double* out);
/* Same into device memory. */
int32_t gsph_get_field_device(gsph_ctx* ctx, int32_t field, double* out);
/* Write results into host records laid out as for gsph_set_particles_aos: only the output
 * fields, and only those computed since the last import (h, u, rho, invomega, zeta,
 * hfactor, hrangesqd, pressure, sound after an h solve; a, atree, gpot, gpot_hydro, dudt,
 * div_v after a force pass); every other byte of the records is left as the caller has it.
 * With flags, only the active particles' fields are written, and levelneib of every
 * particle becomes max(its current value in the record, the neighbour levels the last
 * force pass found), as the reference's force loops update it (MainLoop zeroes levelneib of
 * active particles before the force pass, Sph::ZeroAccelerations, src/Hydrodynamics/Sph.cpp:
 * 126-140).  The force outputs are stored, not added: MainLoop zeroes them for active
 * particles before every force pass (SphSimulation.cpp:646), so storing equals the
 * reference's accumulation.  Page-locked records are written in place by a kernel; other
 * records through a compact device buffer and a host loop. */
int32_t gsph_get_particles_aos(gsph_ctx* ctx, void* base, int64_t n, int64_t stride,
                               const gsph_field_offsets* off);
int32_t gsph_get_stats(gsph_ctx* ctx, gsph_stats* out);

/* ---- verification (the reference's VERIFY_ALL checks, HydroTree.cpp:1900-1985) ----------- */
/* Enable recording of interaction lists in the next force pass (max_sph entries per
 * particle).  Costs atomics; for tests only. */
int32_t gsph_set_recording(gsph_ctx* ctx, int32_t enable, int32_t max_sph);
/* SPH neighbour lists of the last recorded force pass, input ids, CSR layout:
 * offsets[n+1], ids[offsets[n]].  Call with ids == NULL to get the total count. */
int64_t gsph_get_sph_neighbours(gsph_ctx* ctx, int64_t* offsets, int32_t* ids);
/* Direct-sum partners per particle as (count, order-independent 64-bit hash of input
 * ids), and multipole cells per leaf cell as (count, hash of depth-first cell ids). */
int32_t gsph_get_direct_summary(gsph_ctx* ctx, int64_t* counts, uint64_t* hashes);
int32_t gsph_get_cell_summary(gsph_ctx* ctx, int32_t* leaf_cells, int64_t* counts, uint64_t* hashes);
/* Full lists (tests at small N): with recording on, also keep up to max_direct direct-sum
 * partners (input ids) per particle and up to max_cells multipole cells (depth-first ids)
 * per leaf cell in the next force passes; 0, 0 stops.  The getters return CSR arrays —
 * per particle in input order, per leaf in the leaf order of gsph_get_cell_summary — and
 * with ids == NULL the total count. */
int32_t gsph_set_list_recording(gsph_ctx* ctx, int32_t max_direct, int32_t max_cells);
int64_t gsph_get_direct_lists(gsph_ctx* ctx, int64_t* offsets, int32_t* ids);
int64_t gsph_get_cell_lists(gsph_ctx* ctx, int64_t* offsets, int32_t* cells);
/* The KD-tree: per depth-first cell N, and leaf membership as input ids in slot order
 * (slot s holds input id order[s]; leaf cell c holds slots [first[c], first[c]+N[c])). */
int32_t gsph_get_tree(gsph_ctx* ctx, int32_t* cell_n, int32_t* cell_first, int32_t* order,
                      double* cell_data /* ncell x 31, layout of oracle cells */);

/* ---- autotuning ---------------------------------------------------------------------------
 * No counterpart in the reference (whose Nleafmax is a fixed run parameter).  Three knobs
 * set how the pair kernels map a leaf cell onto the GPU:
 *   nleafmax      leaf size: particles per leaf cell, hence per warp of the pair kernels,
 *                 the tree depth and the length of every interaction list;
 *   near_depth    the near-list depth (leaf cells, 64..256) a force warp holds in shared
 *                 memory; a leaf whose near list is deeper goes to the 8-warp kernel, so
 *                 this sets how many warps work on one cell;
 *   cell_depth    the multipole-list tile (64..512 cells) a force warp consumes per flush;
 *   gather_depth  the density gather-list depth (64..256 leaf cells) a warp holds; deeper
 *                 leaves go to the per-particle kernel (one warp per particle).
 * Depths apply to the mixed form; 0 selects the compiled maximum.  Changing nleafmax keeps
 * the imported particles (structure-of-arrays imports only) and rebuilds nothing until the
 * next step; every value is a valid reference configuration, results differ between leaf
 * sizes only as the reference's own results do. */
typedef struct gsph_tuning {
  int32_t nleafmax, near_depth, cell_depth, gather_depth;
} gsph_tuning;
int32_t gsph_get_tuning(gsph_ctx* ctx, gsph_tuning* out);
int32_t gsph_set_tuning(gsph_ctx* ctx, const gsph_tuning* tuning);
/* Times `steps` graph-replayed steps of the imported particles for candidate tunings — a
 * coordinate search: leaf sizes 4, 6, 8, 12, 16, then each depth over its range — and keeps
 * the fastest.  tried / ms (capacity max_tried, may be NULL) receive every candidate and
 * its time per step; *ntried their count.  The context's graphs and any KDK integration are
 * reset; results of the last step are those of the last candidate. */
int32_t gsph_autotune(gsph_ctx* ctx, int32_t steps, gsph_tuning* best, gsph_tuning* tried, double* ms,
                      int32_t max_tried, int32_t* ntried);

/* ---- allocation-free KD-tree ordering --------------------------------------------------- */
/* No counterpart in the reference: an extra entry point for callers that cannot allocate
 * device memory — e.g. a host code whose device memory is all owned by its own pool
 * allocator, or a time-critical loop that cannot afford cudaMalloc's implicit device
 * synchronisation.  It computes the leaf order of the reference KD-tree (the slot order
 * gsph_build_tree produces: order[s] = input index of slot s) for n <= GSPH_NOALLOC_MAX_N
 * particles whose x, y, z, h are device arrays, writing n int32 to the device array
 * order.  Work is enqueued on `stream` (a cudaStream_t, NULL for the legacy default
 * stream) and the call returns without waiting for it.
 *   Memory: no cudaMalloc/cudaFree or other allocating call.  Scratch is one fixed
 *   ~2.6 MiB device array inside the library, held by every GPU that loads the library
 *   until the process exits.  All calls on a device share it, so calls whose work
 *   overlaps on the GPU race; serialise them (one stream, or events).  Each call fully
 *   rewrites the scratch it reads, so nothing left by a previous call leaks into a result.
 *   Set-up: the first call on each device (with that device current) looks up the
 *   array's device address and the SM count; make that first call before any stream
 *   capture.  The address is cached per device for the process: it belongs to the context
 *   current at that first call (the primary context), so do not use this entry point after
 *   cudaDeviceReset or with another context current on that device.
 *   Errors: a CUDA error left pending by the caller's earlier work makes the call return
 *   GSPH_ERR_CUDA before it launches anything (the error is left for the caller to read);
 *   a launch failure of this call's own work returns GSPH_ERR_CUDA.
 *   Limits: 1 <= n <= GSPH_NOALLOC_MAX_N and a tree of at most 13 levels
 *   (Nleafmax * 2^13 >= n).  Larger requests return GSPH_ERR_CAPACITY; bad pointers or
 *   sizes GSPH_ERR_INVALID; CUDA failures GSPH_ERR_CUDA. */
#define GSPH_NOALLOC_MAX_N 32768
int32_t gsph_kdtree_order_noalloc(const double* x, const double* y, const double* z,
                                  const double* h, int32_t n, int32_t nleafmax, int32_t* order,
                                  void* stream);

#ifdef __cplusplus
}
#endif

#endif /* GSPH_GB300_H_ */
