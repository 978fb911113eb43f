// Star-gas gravitational coupling.  FP64, except gas <- stars in the mixed form (FP32
// pair arithmetic on hi + lo float positions, like the form's other pair terms).
//
//  gas <- stars   GradhSph::ComputeStarGravForces (src/GradhSph/GradhSph.cpp:698-743), run
//                 inside the gas force passes after gpot_hydro is taken
//                 (src/GradhSph/GradhSphTree.cpp:385-391, :596-606).
//  star <- gas    HydroTree::UpdateAllStarGasForces (src/Tree/HydroTree.cpp:551-654): a walk
//                 of the gas tree per star (Tree::ComputeStarGravityInteractionList,
//                 src/Tree/Tree.cpp:747-885), kernel-softened terms for the particles of
//                 near leaves and Newtonian terms for the rest
//                 (NbodyHermite4::CalculateDirectHydroForces, src/Nbody/NbodyHermite4.cpp:151-245),
//                 multipole terms for accepted cells (ComputeCellQuadrupoleForces,
//                 src/Headers/NeighbourSearch.h:457-475).
//
// Stars are few (tens), so the gas <- star pass is one thread per gas particle with the
// stars staged in shared memory, and the star <- gas pass is one warp per star.
#include "gsph_walk.cuh"
#include "kernels.cuh"
#include "mixed_state.cuh"
#include "stars.cuh"

namespace gsph {
namespace {

constexpr int kStarChunk = 256;

__global__ void __launch_bounds__(256) k_gas_from_stars(Particles p, StarSet s) {
  __shared__ double sd[8][kStarChunk];
  const int n = p.n;
  for (int base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
    const int slot = base + threadIdx.x;
    const bool mine = slot < n && is_active(p, slot);
    double xi = 0, yi = 0, zi = 0, hi = 1;
    if (mine) { xi = p.x[slot]; yi = p.y[slot]; zi = p.z[slot]; hi = p.h[slot]; }
    double ax = 0.0, ay = 0.0, az = 0.0, pot = 0.0;
    for (int c0 = 0; c0 < s.n; c0 += kStarChunk) {
      const int cn = min(kStarChunk, s.n - c0);
      __syncthreads();
      for (int q = threadIdx.x; q < cn; q += blockDim.x) {
        sd[0][q] = s.x[c0 + q]; sd[1][q] = s.y[c0 + q]; sd[2][q] = s.z[c0 + q];
        sd[3][q] = s.m[c0 + q]; sd[4][q] = s.h[c0 + q];
      }
      __syncthreads();
      if (mine) {
        for (int j = 0; j < cn; j++) {
          const double dx = __dsub_rn(sd[0][j], xi), dy = __dsub_rn(sd[1][j], yi), dz = __dsub_rn(sd[2][j], zi);
          const double drsqd = __dadd_rn(dot3_rn(dx, dy, dz), kSmall);
          const double drmag = sqrt(drsqd);
          const double invdrmag = 1.0 / drmag;
          const double invhmean = 2.0 / (hi + sd[4][j]);
          const double ms = sd[3][j];
          const double paux = ms * invhmean * invhmean * m4_wgrav(drmag * invhmean) * invdrmag;
          ax += paux * dx; ay += paux * dy; az += paux * dz;
          pot += ms * invhmean * m4_wpot(drmag * invhmean);
        }
      }
    }
    if (mine) {
      p.gpot_hydro[slot] = p.gpot[slot];
      p.agx[slot] += ax; p.agy[slot] += ay; p.agz[slot] += az;
      p.ax[slot] += ax; p.ay[slot] += ay; p.az[slot] += az;
      p.gpot[slot] += pot;
    }
  }
}

// Mixed form: the same sums in single precision (positions as hi + lo float pairs, one
// reciprocal per pair and no other division), added to the fp64 accumulators.
__global__ void __launch_bounds__(256) k_gas_from_stars_f(Particles p, MixedParticles mp, StarSet s) {
  __shared__ float4 shi[kStarChunk], slo[kStarChunk];
  const int n = p.n;
  for (int base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
    const int slot = base + threadIdx.x;
    const bool mine = slot < n && is_active(p, slot);
    float4 ph = make_float4(0.f, 0.f, 0.f, 0.f), pl = ph;
    float hi = 1.0f;
    if (mine) { ph = mp.pos_hi[slot]; pl = mp.pos_lo[slot]; hi = (float) p.h[slot]; }
    float ax = 0.0f, ay = 0.0f, az = 0.0f, pot = 0.0f;
    for (int c0 = 0; c0 < s.n; c0 += kStarChunk) {
      const int cn = min(kStarChunk, s.n - c0);
      __syncthreads();
      for (int q = threadIdx.x; q < cn; q += blockDim.x) { shi[q] = s.fhi[c0 + q]; slo[q] = s.flo[c0 + q]; }
      __syncthreads();
      if (mine) {
        for (int j = 0; j < cn; j++) {
          const float4 sh = shi[j], sl = slo[j];
          const float dx = (sh.x - ph.x) + (sl.x - pl.x);
          const float dy = (sh.y - ph.y) + (sl.y - pl.y);
          const float dz = (sh.z - ph.z) + (sl.z - pl.z);
          const float r2 = dx * dx + dy * dy + dz * dz + 1.0e-20f;
          const float invdrmag = rsqrtf(r2);
          const float drmag = r2 * invdrmag;
          const float hsum = hi + sl.w;
          const float invhmean = __fdividef(2.0f, hsum);
          // 1/s = hmean / |r|
          float w1, wg, wp;
          m4f_w1_grav_pot(drmag * invhmean, 0.5f * hsum * invdrmag, w1, wg, wp);
          const float paux = sh.w * invhmean * invhmean * wg * invdrmag;
          ax += paux * dx; ay += paux * dy; az += paux * dz;
          pot += sh.w * invhmean * wp;
        }
      }
    }
    if (mine) {
      p.gpot_hydro[slot] = p.gpot[slot];
      p.agx[slot] += ax; p.agy[slot] += ay; p.agz[slot] += az;
      p.ax[slot] += ax; p.ay[slot] += ay; p.az[slot] += az;
      p.gpot[slot] += pot;
    }
  }
}

constexpr int kStarWarps = 4;
constexpr int kStarStack = 1024;
constexpr int kStarList = 256;

__device__ __forceinline__ double wsum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}

// One warp per star.  ppl: lanes per leaf (power of two >= the largest leaf).
__global__ void __launch_bounds__(kStarWarps * 32)
k_stars_from_gas(Tree t, Particles p, StarSet s, SphParams prm, DeviceCounters cnt, int ppl) {
  __shared__ int s_stack[kStarWarps][kStarStack];
  __shared__ int s_list[kStarWarps][3][kStarList];
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int star = blockIdx.x * kStarWarps + wib;
  if (star >= s.n) return;
  const double rs[3] = {s.x[star], s.y[star], s.z[star]};
  const double vs[3] = {s.vx[star], s.vy[star], s.vz[star]};
  const double hs = s.h[star];
  // 0.5 hrangemax + rmax + 0.5 kernrange hmax with hrangemax = kernrange h_star (Tree.cpp:797-801)
  const double half_hrange = __dmul_rn(0.5, __dmul_rn(kKernRange, hs));
  const double half_kr = 0.5 * kKernRange;
  const bool quad = prm.multipole == 1;
  double a[3] = {0.0, 0.0, 0.0}, ad[3] = {0.0, 0.0, 0.0}, pot = 0.0;

  auto decide = [&](int node, int level) -> int {
    const CellGeom g = t.geom[node];
    const double dx = __dsub_rn(g.rcell[0], rs[0]), dy = __dsub_rn(g.rcell[1], rs[1]),
                 dz = __dsub_rn(g.rcell[2], rs[2]);
    const double drsqd = dot3_rn(dx, dy, dz);
    const double reach = __dadd_rn(__dadd_rn(half_hrange, g.rmax), __dmul_rn(half_kr, g.hmax));
    const int nn = t.cell_n[node];
    if (drsqd < __dmul_rn(reach, reach)) {
      if (level < t.ltot) return kOpen;
      return nn > 0 ? kEmitA : kSkip;
    }
    if (nn > 0 && drsqd > g.cdistsqd) return (level == t.ltot && nn == 1) ? kEmitB : kEmitC;
    if (nn > 0 && drsqd <= g.cdistsqd) return level < t.ltot ? kOpen : kEmitB;
    return kSkip;
  };
  auto tag = [](int node, int) { return node; };
  WarpLists L{s_list[wib][0], s_list[wib][1], s_list[wib][2], 0, 0, 0, kStarList};
  const int per = 32 / ppl;
  auto consume = [&]() {
    // kernel-softened terms for the particles of near leaves
    for (int e0 = 0; e0 < L.na; e0 += per) {
      const int e = e0 + lane / ppl, q = lane % ppl;
      if (e >= L.na) continue;
      const int node = L.a[e];
      if (q >= t.cell_n[node]) continue;
      const int j = t.cell_first[node] + q;
      const double dr[3] = {__dsub_rn(p.x[j], rs[0]), __dsub_rn(p.y[j], rs[1]), __dsub_rn(p.z[j], rs[2])};
      const double dv[3] = {__dsub_rn(p.vx[j], vs[0]), __dsub_rn(p.vy[j], vs[1]), __dsub_rn(p.vz[j], vs[2])};
      const double drsqd = dot3_rn(dr[0], dr[1], dr[2]);
      const double drmag = sqrt(drsqd);
      const double invdrmag = 1.0 / drmag;
      const double invhmean = 2.0 / (hs + p.h[j]);
      const double mj = p.m[j];
      const double drdt = (dv[0] * dr[0] + dv[1] * dr[1] + dv[2] * dr[2]) * invdrmag;
      const double paux = mj * invhmean * invhmean * m4_wgrav(drmag * invhmean) * invdrmag;
      // powf(invhmean, ndim) in the reference: the cube of the float value, rounded once
      // to float (the double product of three floats is exact to 2^-53)
      const double ihf = (double) (float) invhmean;
      const double wkern = m4_w0(drmag * invhmean) * (double) (float) (ihf * ihf * ihf);
      for (int k = 0; k < 3; k++) {
        a[k] += paux * dr[k];
        ad[k] += paux * dv[k] - 3.0 * paux * drdt * invdrmag * dr[k] +
                 2.0 * kTwoPi * mj * drdt * wkern * invdrmag * dr[k];
      }
      pot += mj * invhmean * m4_wpot(drmag * invhmean);
    }
    // Newtonian terms for the particles of opened leaves (and far single-particle leaves)
    for (int e0 = 0; e0 < L.nb; e0 += per) {
      const int e = e0 + lane / ppl, q = lane % ppl;
      if (e >= L.nb) continue;
      const int node = L.b[e];
      if (q >= t.cell_n[node]) continue;
      const int j = t.cell_first[node] + q;
      const double dr[3] = {__dsub_rn(p.x[j], rs[0]), __dsub_rn(p.y[j], rs[1]), __dsub_rn(p.z[j], rs[2])};
      const double dv[3] = {__dsub_rn(p.vx[j], vs[0]), __dsub_rn(p.vy[j], vs[1]), __dsub_rn(p.vz[j], vs[2])};
      const double drsqd = dot3_rn(dr[0], dr[1], dr[2]);
      const double drmag = sqrt(drsqd);
      const double invdrmag = 1.0 / drmag;
      const double mj = p.m[j];
      const double drdt = (dv[0] * dr[0] + dv[1] * dr[1] + dv[2] * dr[2]) * invdrmag;
      const double inv3 = invdrmag * invdrmag * invdrmag;
      for (int k = 0; k < 3; k++) {
        a[k] += mj * dr[k] * inv3;
        ad[k] += mj * inv3 * (dv[k] - 3.0 * drdt * invdrmag * dr[k]);
      }
      pot += mj * invdrmag;
    }
    // accepted cells: multipole terms about the star
    for (int e = lane; e < L.nc; e += 32) {
      const CellMoment c = t.mom[L.c[e]];
      if (quad) {
        const double dx = rs[0] - c.r[0], dy = rs[1] - c.r[1], dz = rs[2] - c.r[2];
        const double drsqd = dx * dx + dy * dy + dz * dz + kSmall;
        const double invdrsqd = 1.0 / drsqd;
        const double invdrmag = sqrt(invdrsqd);
        const double invdr5 = invdrsqd * invdrsqd * invdrmag;
        const double mon = c.m * invdrsqd * invdrmag;
        a[0] -= mon * dx; a[1] -= mon * dy; a[2] -= mon * dz;
        const double* q = c.q;
        const double qzz = -(q[0] + q[2]);
        const double qscalar = q[0] * dx * dx + q[2] * dy * dy + qzz * dz * dz +
                               2.0 * (q[1] * dx * dy + q[3] * dx * dz + q[4] * dy * dz);
        const double qfactor = 2.5 * qscalar * invdr5 * invdrsqd;
        a[0] += (q[0] * dx + q[1] * dy + q[3] * dz) * invdr5 - qfactor * dx;
        a[1] += (q[1] * dx + q[2] * dy + q[4] * dz) * invdr5 - qfactor * dy;
        a[2] += (q[3] * dx + q[4] * dy + qzz * dz) * invdr5 - qfactor * dz;
        pot += c.m * invdrmag + 0.5 * qscalar * invdr5;
      } else {
        const double dx = c.r[0] - rs[0], dy = c.r[1] - rs[1], dz = c.r[2] - rs[2];
        const double drsqd = dx * dx + dy * dy + dz * dz + kSmall;
        const double invdrsqd = 1.0 / drsqd;
        const double invdrmag = sqrt(invdrsqd);
        pot += c.m * invdrmag;
        const double f = c.m * invdrsqd * invdrmag;
        a[0] += f * dx; a[1] += f * dy; a[2] += f * dz;
      }
    }
    __syncwarp();
  };
  const bool ok = warp_walk(0, t.ltot, t.cell_level, s_stack[wib], kStarStack, L, decide, tag, consume);
  consume();
  if (!ok && lane == 0) atomicOr(cnt.status, (unsigned) kStatusStackOverflow);
  for (int k = 0; k < 3; k++) { a[k] = wsum(a[k]); ad[k] = wsum(ad[k]); }
  pot = wsum(pot);
  if (lane == 0) {
    s.ax[star] = a[0]; s.ay[star] = a[1]; s.az[star] = a[2];
    s.adotx[star] = ad[0]; s.adoty[star] = ad[1]; s.adotz[star] = ad[2];
    s.gpot[star] = pot;
  }
}

}  // namespace

int launch_gas_from_stars(const Particles& p, const StarSet& s, cudaStream_t st) {
  if (s.n <= 0) return 0;
  const int blocks = std::max(1, std::min((p.n + 255) / 256, 152 * 8));
  k_gas_from_stars<<<blocks, 256, 0, st>>>(p, s);
  return 1;
}

int launch_gas_from_stars_mixed(const Particles& p, const MixedParticles& mp, const StarSet& s, cudaStream_t st) {
  if (s.n <= 0) return 0;
  const int blocks = std::max(1, std::min((p.n + 255) / 256, 152 * 8));
  k_gas_from_stars_f<<<blocks, 256, 0, st>>>(p, mp, s);
  return 1;
}

int launch_stars_from_gas(const Tree& t, const Particles& p, const StarSet& s, const SphParams& prm,
                          const DeviceCounters& cnt, int max_leaf, cudaStream_t st) {
  if (s.n <= 0) return 0;
  int ppl = 1;
  while (ppl < max_leaf) ppl <<= 1;
  k_stars_from_gas<<<(s.n + kStarWarps - 1) / kStarWarps, kStarWarps * 32, 0, st>>>(t, p, s, prm, cnt, ppl);
  return 1;
}

}  // namespace gsph
