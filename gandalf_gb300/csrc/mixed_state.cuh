// Single-precision mirrors used by the mixed-precision form.
//
// Positions are held as unevaluated float sums x = hi + lo (hi = (float) x,
// lo = (float) (x - hi)); the difference of two such positions,
// (hi_j - hi_i) + (lo_j - lo_i), carries a relative error of a few float ulps of the
// separation itself, which is what coordinates relative to a cell centre give.  All
// membership decisions (tree walk, SPH neighbour test) are first made in float with a
// relative margin and re-made in fp64, exactly as the reference computes them, whenever
// the float result falls inside the margin.
#pragma once
#include "gsph_state.cuh"

namespace gsph {

struct MixedParticles {
  float4* pos_hi;   // x_hi y_hi z_hi m
  float4* pos_lo;   // x_lo y_lo z_lo, hrangesqd (0 until the h solve)
  float4* vel;      // vx vy vz h
  float4* hyd;      // 1/h  P*invomega/rho^2  1/rho  sound
  float4* aux;      // hfactor zeta hrangesqd 0
};

struct MixedCells {
  float4* geo_hi;   // rcell_hi xyz, rmax
  float4* geo_lo;   // rcell_lo xyz, hmax (after the h solve)
  float4* meta;     // cdistsqd, cell_n, level and cell_first (int bits): one load per walk decision
  float4* com_hi;   // com_hi xyz, m
  float4* com_lo;   // com_lo xyz, q4
  float4* quad;     // q0 q1 q2 q3
  float4* bbmin;    // bounding box rounded outwards; w: cell_n (int bits)
  float4* bbmax;    // w: (cell_first << 5) | level (int bits)
  float4* hbmin;    // smoothing-volume box rounded outwards
  float4* hbmax;
};

// Leaves the warp-per-leaf kernels hand over to the heavy-leaf kernels.
struct HeavyList {
  int* leaves;      // leaf indices
  int* count;       // device counter
};

int mixed_max_particles();   // the most particles the mixed form's list words address

void launch_mixed_prep_build(const Tree& t, const Particles& p, const MixedParticles& mp,
                             const MixedCells& mc, cudaStream_t st);
void launch_mixed_prep_hydro(const Tree& t, const Particles& p, const MixedParticles& mp,
                             const MixedCells& mc, cudaStream_t st);

}  // namespace gsph
