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

// The same sum in single precision for the mixed form, positions as hi + lo float pairs;
// stars j0, j0 + stride, ... (the lanes of a particle share the stars and add up).
__device__ __forceinline__ float star_zeta_part_f(const StarSet& s, float4 ph, float4 pl, float h, int j0,
                                                  int stride) {
  float z = 0.0f;
  for (int j = j0; j < s.n; j += stride) {
    const float4 sh = s.fhi[j], sl = s.flo[j];
    const float ih = __fdividef(2.0f, h + sl.w);
    const float ihsqd = ih * ih;
    const float dx = (sh.x - ph.x) + (sl.x - pl.x);
    const float dy = (sh.y - ph.y) + (sl.y - pl.y);
    const float dz = (sh.z - ph.z) + (sl.z - pl.z);
    const float ssqd = (dx * dx + dy * dy + dz * dz) * ihsqd;
    const float sv = ssqd > 0.0f ? ssqd * rsqrtf(ssqd) : 0.0f;
    z += sh.w * ihsqd * m4f_wzeta(sv);
  }
  return z;
}

int launch_gas_from_stars(const Particles& p, const StarSet& s, cudaStream_t st);
struct MixedParticles;
int launch_gas_from_stars_mixed(const Particles& p, const MixedParticles& mp, const StarSet& s, cudaStream_t st);
int launch_stars_from_gas(const Tree& t, const Particles& p, const StarSet& s, const SphParams& prm,
                          const DeviceCounters& cnt, int max_leaf, cudaStream_t st);

}  // namespace gsph
