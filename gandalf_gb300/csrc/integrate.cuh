// Leapfrog KDK integration with hierarchical block timesteps, on the device.
//
// The integer-time state of the reference's Simulation (n, nresync, level_max, level_step,
// timestep, dt_max, t; src/Headers/Simulation.h:187-215) lives in one device record so
// that a whole sequence of steps runs without host round trips (and can be captured into
// one CUDA graph).  Per-particle integration state is kept in input order; the solved
// fields of particles that are not active in a step persist in input order too and are
// gathered into leaf order after each tree build.
#pragma once
#include "gsph_state.cuh"

namespace gsph {

struct KdkGlobal {
  int n, nresync, level_max, level_step, Nsteps;
  int activecount;            // particles CheckTimesteps made active in the last pass
  int level_max_new;          // reduction: largest particle level
  int nfactor_up, nfactor_down;
  int resync;                 // the last block-timestep call took the resynchronisation branch
  int bt_count;               // particles listed for a new timestep (KdkState::bt_list)
  unsigned status;            // KdkStatus bits
  double t, timestep, dt_max, timestep_old;
  unsigned long long dtmin_bits;     // atomicMin over the bits of positive doubles
  unsigned long long active_updates; // active particles summed over all passes and steps
  unsigned long long repeat_passes;  // CheckTimesteps repeat passes executed
};

enum KdkStatus : unsigned {
  kKdkTimestepInvalid = 1u,   // Timestep() out of range ("Hydro timestep too large")
  kKdkNotSettled = 2u,        // CheckTimesteps still activating particles after the last pass
};

struct KdkParams {
  int nlevels, level_diff_max, energy_integration, periodic;
  double courant_mult, accel_mult, energy_mult;
  double boxmin[3], boxmax[3], boxsize[3];
};

// Per-particle state in input order.  keep[] are the persistent solved fields, laid out
// like the leaf-order fields they mirror (rho invomega zeta hfactor hrangesqd pressure sound
// ax ay az agx agy agz gpot dudt div_v gpot_hydro).
constexpr int kKeep = 17;
constexpr int kKSound = 6, kKAX = 7, kKAY = 8, kKAZ = 9, kKDudt = 14, kKDivV = 15;
struct KdkState {
  int n;
  double *x, *y, *z, *vx, *vy, *vz, *u, *h;   // current values (the tree build's inputs)
  double *r0[3], *v0[3], *a0[3];
  double *u0, *dudt0, *dt, *dt_next, *tlast;
  int *nlast, *nstep, *level, *levelneib;
  unsigned char* flags;                        // kFlagActive | kFlagEndStep
  int* bt_list;                                // particles whose timestep is computed this step
  double* keep[kKeep];
};
constexpr unsigned char kFlagActive = 1, kFlagEndStep = 2;
constexpr unsigned char kFlagTouched = 4;   // active in some pass of the current step
// keep[] fields an inactive particle's neighbours read in a pass (rho invomega zeta hfactor
// hrangesqd); pressure and sound are recomputed for every particle before each force pass
constexpr int kKeepNeighbour = 5;
constexpr int kKPressure = 5;

// Leaf-order views the gather / scatter kernels fill.
struct KdkLeaf {
  int n;
  const int* id;
  const int* slot_of;      // slot of each input index: scatters run in input order (coalesced
                           // stores, random loads instead of random stores)
  double* f[kKeep];        // leaf-order fields matching keep[]
  double *h, *u;           // leaf-order h and u
  unsigned char* active;
  int *level, *lvn;
};

void launch_kdk_begin(KdkGlobal* g, cudaStream_t st);
void launch_kdk_advance(const KdkState& s, const KdkParams& kp, KdkGlobal* g, cudaStream_t st);
void launch_kdk_gather(const KdkState& s, const KdkLeaf& l, KdkGlobal* g, cudaStream_t st);
void launch_kdk_scatter(const KdkState& s, const KdkLeaf& l, cudaStream_t st);
void launch_kdk_refresh(const KdkState& s, const KdkLeaf& l, KdkGlobal* g, cudaStream_t st);
void launch_kdk_scatter_lvn(const KdkState& s, const KdkLeaf& l, cudaStream_t st);
void launch_kdk_scatter_fields(const KdkState& s, const KdkLeaf& l, cudaStream_t st);
void launch_kdk_check(const KdkState& s, const KdkParams& kp, KdkGlobal* g, bool last_pass, cudaStream_t st);
void launch_kdk_timesteps(const KdkState& s, const KdkParams& kp, KdkGlobal* g, cudaStream_t st);
void launch_kdk_end(const KdkState& s, const KdkParams& kp, KdkGlobal* g, cudaStream_t st);
void launch_kdk_setup_state(const KdkState& s, KdkGlobal* g, cudaStream_t st);
void launch_kdk_setup_finish(const KdkState& s, cudaStream_t st);
void launch_kdk_thermal(const Particles& p, const SphParams& prm, cudaStream_t st);
// Sets a graph conditional to (particles were activated by the last CheckTimesteps).
void launch_kdk_set_cond(cudaGraphConditionalHandle h, const KdkGlobal* g, cudaStream_t st);

}  // namespace gsph
