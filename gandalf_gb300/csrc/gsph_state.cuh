// Device-side state shared by the kernels of one context (plain pointers, passed by value).
#pragma once
#include "gsph_common.cuh"

namespace gsph {

// Star particles (NbodyParticle r, v, m, h; device arrays of n each) and the star <- gas
// results the star walk writes.
struct StarSet {
  int n;
  const double *x, *y, *z, *vx, *vy, *vz, *m, *h;
  double *ax, *ay, *az, *adotx, *adoty, *adotz, *gpot;
};

struct SphParams {
  double h_fac, h_converge, alpha_visc, beta_visc, gamma_eos, temp0, mu_bar, thetamaxsqd;
  double boxmin[3], boxmax[3], boxsize[3], boxhalf[3];
  int eos;          // 0 adiabatic energy equation, 1 isothermal
  int periodic;     // 0 open, 1 periodic in x, y and z
  int multipole;    // 0 monopole, 1 quadrupole
  int self_gravity;
  StarSet stars;    // n = 0: no stars
};

// Particles in leaf order (slot = position in the leaf-ordered arrays).
struct Particles {
  int n;
  const int* id;              // input index of each slot
  double *x, *y, *z, *vx, *vy, *vz, *m, *u, *h;
  double* h0;                 // h when the tree was built (ghost ranges, cell stock)
  double *rho, *invomega, *zeta, *hfactor, *hrangesqd, *pressure, *sound;
  double *ax, *ay, *az, *agx, *agy, *agz, *gpot, *dudt, *div_v;
  double* gpot_hydro;         // gpot before the star terms (written only with stars)
};

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
  unsigned* climb;            // per-cell arrival counters for bottom-up passes
};

}  // namespace gsph
