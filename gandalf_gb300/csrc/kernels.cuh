// Launchers of the per-leaf-cell kernels (density.cu, forces.cu).
#pragma once
#include "gsph_state.cuh"

namespace gsph {

// Device-side counters and status word, zeroed by the host before a step.
struct DeviceCounters {
  unsigned* status;                    // StatusBits, or-ed by kernels
  unsigned long long* density_pairs;   // pair evaluations inside the kernel support
  unsigned long long* hydro_pairs;     // SPH pairs (hydro or hydro + softened gravity)
  unsigned long long* direct_pairs;    // Newtonian particle-particle terms
  unsigned long long* cell_pairs;      // particle-cell multipole terms
  unsigned long long* exact_checks;    // mixed form: membership tests resolved in fp64
  // optional recording of interaction lists (verification only; record == 0 skips it)
  int record;
  int rec_max;                         // SPH ids kept per particle
  int* rec_sph_cnt;                    // per slot
  int* rec_sph_ids;                    // slot * rec_max
  unsigned long long* rec_dir_cnt;     // per slot
  unsigned long long* rec_dir_hash;    // per slot: sum of mix64(input id)
  unsigned long long* rec_cell_cnt;    // per leaf index
  unsigned long long* rec_cell_hash;   // per leaf index: sum of mix64(cell id)
  // optional full lists (nullptr: not kept): direct-sum partners per slot (input ids) and
  // multipole cells per leaf index (depth-first ids), rec_*_max entries each
  int rec_dir_max, rec_cell_max;
  int *rec_dir_n, *rec_dir_ids;
  int *rec_cell_n, *rec_cell_ids;
};

__device__ __forceinline__ void rec_direct_id(const DeviceCounters& c, int slot, int id) {
  if (!c.rec_dir_ids) return;
  const int k = atomicAdd(&c.rec_dir_n[slot], 1);
  if (k < c.rec_dir_max) c.rec_dir_ids[(size_t) slot * c.rec_dir_max + k] = id;
}
__device__ __forceinline__ void rec_cell_id(const DeviceCounters& c, int leaf, int cell) {
  if (!c.rec_cell_ids) return;
  const int k = atomicAdd(&c.rec_cell_n[leaf], 1);
  if (k < c.rec_cell_max) c.rec_cell_ids[(size_t) leaf * c.rec_cell_max + k] = cell;
}

__host__ __device__ __forceinline__ unsigned long long mix64(unsigned long long x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

struct MixedParticles;
struct MixedCells;
struct HeavyList;

// mixed-precision form (mixed.cu); each returns the number of kernels it launched
int launch_density_mixed(const Tree& t, const Particles& p, const MixedParticles& mp, const MixedCells& mc,
                         const SphParams& prm, const DeviceCounters& cnt, const HeavyList& heavy,
                         const HeavyList& wide, int lanes_per_particle, int max_leaf, cudaStream_t st);
int launch_all_forces_mixed(const Tree& t, const Particles& p, const MixedParticles& mp, const MixedCells& mc,
                            const SphParams& prm, const DeviceCounters& cnt, const HeavyList& heavy,
                            int lanes_per_particle, int max_leaf, cudaStream_t st);
int launch_hydro_mixed(const Tree& t, const Particles& p, const MixedParticles& mp, const MixedCells& mc,
                       const SphParams& prm, const DeviceCounters& cnt, int lanes_per_particle, cudaStream_t st);

// FP64 h solve; leaves whose gather list does not fit one warp go to a heavy-leaf kernel
// through `heavy` (count zeroed here).  `next` is a leaf counter (zeroed here) and
// `scratch` holds density_fp64_scratch_entries() double2.  Launches two kernels.
size_t density_fp64_scratch_entries();
void launch_density(const Tree& t, const Particles& p, const SphParams& prm, const DeviceCounters& cnt,
                    const HeavyList& heavy, int lanes_per_particle, int* next, double2* scratch, cudaStream_t st);
void launch_hydro_forces(const Tree& t, const Particles& p, const SphParams& prm,
                         const DeviceCounters& cnt, int lanes_per_particle, cudaStream_t st);
void launch_all_forces(const Tree& t, const Particles& p, const SphParams& prm,
                       const DeviceCounters& cnt, int lanes_per_particle, cudaStream_t st);

}  // namespace gsph
