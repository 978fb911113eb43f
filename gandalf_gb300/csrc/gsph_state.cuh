// Device-side state shared by the kernels of one context (plain pointers, passed by value).
#pragma once
#include "gsph_common.cuh"

namespace gsph {

// Star particles (NbodyParticle r, v, m, h; device arrays of n each) and the star <- gas
// results the star walk writes.
struct StarSet {
  int n;
  const double *x, *y, *z, *vx, *vy, *vz, *m, *h;
  const float4 *fhi, *flo;   // mixed form: (x_hi y_hi z_hi m), (x_lo y_lo z_lo h)
  double *ax, *ay, *az, *adotx, *adoty, *adotz, *gpot;
};

struct SphParams {
  double h_fac, h_converge, alpha_visc, beta_visc, gamma_eos, temp0, mu_bar, thetamaxsqd;
  double u_iso;     // isothermal specific energy temp0 / (gamma - 1) / mu_bar, evaluated on the host
  double boxmin[3], boxmax[3], boxsize[3], boxhalf[3];
  int eos;          // 0 adiabatic energy equation, 1 isothermal
  int periodic;     // 0 open, 1 periodic in x, y and z
  int multipole;    // 0 monopole, 1 quadrupole
  int self_gravity;
  int compensated;  // mixed form: compensated float sums, lane partials combined in fp64
  // Tuned list depths of the mixed warp-per-leaf kernels (0: the compiled maximum): the
  // near-list depth a force warp keeps before its leaf goes to the 8-warp kernel, the
  // multipole-list depth consumed per flush, and the density gather-list depth before a
  // leaf goes to the per-particle kernel.
  int near_depth, cell_depth, gather_depth;
  // float roundings of alpha_visc, beta_visc * alpha_visc and gamma - 1 for the mixed pair
  // loops, formed on the host: on the device each would be an fp64 multiply or conversion
  // per pair, and GB300 charges an fp64 instruction per warp at 1/64 of the fp32 rate
  float alpha_visc_f, ab_visc_f, gm1_f;
  StarSet stars;    // n = 0: no stars
};

// A tuned depth clamped to [lo, max] (0 selects max).
__host__ __device__ __forceinline__ int tuned_depth(int v, int lo, int max) {
  return v <= 0 ? max : (v < lo ? lo : (v > max ? max : v));
}

// Kahan-compensated float accumulation: s + c carries the sum to about twice float precision
// (the lost low part of each addition is kept in c and fed back into the next one).
__device__ __forceinline__ void kahan_add(float& s, float& c, float v) {
  const float y = __fsub_rn(v, c);
  const float t = __fadd_rn(s, y);
  c = __fsub_rn(__fsub_rn(t, s), y);
  s = t;
}

// Particles in leaf order (slot = position in the leaf-ordered arrays).
struct Particles {
  int n;
  const int* id;              // input index of each slot
  double *x, *y, *z, *vx, *vy, *vz, *m, *u, *h;
  double* h0;                 // h when the tree was built (ghost ranges, cell stock)
  double *rho, *invomega, *zeta, *hfactor, *hrangesqd, *pressure, *sound;
  double *ax, *ay, *az, *agx, *agy, *agz, *gpot, *dudt, *div_v;
  double* gpot_hydro;         // gpot before the star terms (written only with stars)
  double *invh_p, *invrho_p, *fac_p;   // FP64 force pass: 1/h, 1/rho, P Omega^-1 / rho^2 per slot
  // block timesteps (nullptr when every particle is active and levels are not tracked)
  const unsigned char* active;   // per slot: 1 = the h solve and forces are computed
  const int* level;              // per slot: timestep level
  int* lvn;                      // per slot: max level of its SPH neighbours (atomicMax)
};

__device__ __forceinline__ bool is_active(const Particles& p, int slot) { return !p.active || p.active[slot]; }

// Whether the periodic image of particle j shifted by (sx, sy, sz) box lengths exists as a
// ghost: the reference makes ghosts only of particles within ghost_range * kernrange * h of
// the boundary they are copied across, with h as at the tree build (HydroTree.cpp:494-543).
__device__ __forceinline__ bool ghost_exists(const SphParams& prm, const Particles& p, int j, const int* sh) {
  const double lim = __dmul_rn(kGhostRange * kKernRange, p.h0[j]);
  const double r[3] = {p.x[j], p.y[j], p.z[j]};
  for (int k = 0; k < 3; k++) {
    if (sh[k] > 1 || sh[k] < -1) return false;
    if (sh[k] > 0 && !(r[k] < __dadd_rn(prm.boxmin[k], lim))) return false;
    if (sh[k] < 0 && !(r[k] > __dsub_rn(prm.boxmax[k], lim))) return false;
  }
  return true;
}

// levelneib bookkeeping of one SPH pair (i active, j its neighbour; GradhSph.cpp:445-446):
// i takes the largest neighbour level and j the level of i (for a periodic image j is the
// real particle, as NeighbourManager::GetNeibI maps ghosts back, NeighbourManager.h:296-302).
__device__ __forceinline__ void lvn_pair(const Particles& p, int slot_i, int j, int& own) {
  if (!p.level) return;
  own = max(own, p.level[j]);
  atomicMax(&p.lvn[j], p.level[slot_i]);
}
__device__ __forceinline__ void lvn_finish(const Particles& p, int slot, bool mine, int own) {
  if (p.level && mine && own > 0) atomicMax(&p.lvn[slot], own);
}

// Tree topology (static per N) and stocked cell data (depth-first ids).
struct Tree {
  int n, ltot, ncell, nleaf;
  const int* cell_first;      // first slot of each cell
  const int* cell_n;          // particles in each cell
  const unsigned char* cell_level;
  const int* cell_parent;     // -1 for the root
  const int* leaf_cell;       // depth-first id of leaf s (left to right)
  CellGeom* geom;             // rcell, rmax, hmax, cdistsqd
  CellBox* bb;                // tight particle bounding box
  CellBox* hbox;              // bounding box of smoothing volumes
  CellMoment* mom;            // centre of mass, mass, quadrupole
};

}  // namespace gsph
