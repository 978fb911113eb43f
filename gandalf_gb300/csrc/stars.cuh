// Star-gas coupling helpers shared by the density kernels and stars.cu.
#pragma once
#include "kernels.cuh"

namespace gsph {

// SPH-star conservative-gravity zeta term (Hubber et al. 2013) that GradhSph::ComputeH
// adds for every star after the h iteration (src/GradhSph/GradhSph.cpp:282-297, softened
// N-body gravity): sum_s m_s hmean^-2 wzeta(|r_s - r_i| / hmean), 1/hmean = 2/(h_i + h_s).
// Added to the particle's zeta sum before the h_rho_deriv * invomega scaling.
__device__ __forceinline__ double star_zeta_sum(const StarSet& s, double xi, double yi, double zi, double h) {
  double z = 0.0;
  for (int j = 0; j < s.n; j++) {
    const double ih = 2.0 / (h + s.h[j]);
    const double ihsqd = ih * ih;
    const double dx = __dsub_rn(s.x[j], xi), dy = __dsub_rn(s.y[j], yi), dz = __dsub_rn(s.z[j], zi);
    const double ssqd = __dmul_rn(dot3_rn(dx, dy, dz), ihsqd);
    z += s.m[j] * ihsqd * m4_wzeta(sqrt(ssqd));
  }
  return z;
}

int launch_gas_from_stars(const Particles& p, const StarSet& s, cudaStream_t st);
int launch_stars_from_gas(const Tree& t, const Particles& p, const StarSet& s, const SphParams& prm,
                          const DeviceCounters& cnt, int max_leaf, cudaStream_t st);

}  // namespace gsph
