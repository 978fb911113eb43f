// Batched passes over many independent simulations (mixed form).
//
// Every per-leaf device function of the single-simulation kernels takes its simulation's
// tree, particles and parameters as arguments, so one persistent launch can serve the
// leaf cells of all simulations of a batch: each warp (or block, for heavy leaves) takes
// the next item of a device work counter, finds the simulation it belongs to from the
// prefix sums of the simulations' leaf counts, and runs the same per-leaf code on that
// simulation's data.  Leaves of uneven cost balance themselves: a warp that finishes early
// takes the next item.
#pragma once
#include "kernels.cuh"
#include "mixed_state.cuh"

namespace gsph {

// Everything the per-leaf kernels of one simulation read.
struct SimDesc {
  Tree t;
  Particles p;
  MixedParticles mp;
  MixedCells mc;
  SphParams prm;
  DeviceCounters cnt;
  HeavyList heavy;
};

// Work queue over the leaf cells of all simulations (device pointers).
struct BatchQueue {
  int nsim;
  const SimDesc* sims;
  const int* leaf_start;   // nsim + 1 prefix sums of the simulations' leaf counts
  int* heavy_start;        // nsim + 1 prefix sums of the heavy-leaf counts (device-filled)
  int* next;               // work counters: normal density, heavy density, normal forces, heavy forces
  bool record;             // some simulation records its pair lists: the recording kernels run
};

// Each returns the number of kernels it launched.  lpg: lanes per particle, chosen for the
// largest leaf of any simulation of the batch.
int launch_batch_density(const BatchQueue& q, int lpg, cudaStream_t st);
int launch_batch_forces(const BatchQueue& q, bool gravity, int lpg, cudaStream_t st);

}  // namespace gsph
