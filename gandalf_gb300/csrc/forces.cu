// Hydro and hydro + self-gravity force passes, one warp per leaf cell (fp64 form).
//
// Reference drivers: GradhSphTree::UpdateAllSphHydroForces (src/GradhSph/GradhSphTree.cpp:279-435)
// and GradhSphTree::UpdateAllSphForces (:443-657).  Per leaf the warp walks the tree once
// (Tree::ComputeNeighbourAndGhostList, src/Tree/Tree.cpp:561-617, or
// Tree::ComputeGravityInteractionAndGhostList, :627-735) into three shared-memory lists —
// near leaf cells (SPH candidates), direct-sum leaf cells and multipole cells — and
// consumes them whenever one fills.  Group g of LPG lanes owns particle g of the leaf.
//
// Pair membership follows NeighbourManager::TrimNeighbourLists
// (src/Headers/NeighbourManager.h:482-543): j is an SPH neighbour of i when
// |r_ij|^2 < 4 h_i^2 or < 4 h_j^2, computed without fused operations exactly as the
// reference; every other near particle is a Newtonian direct-sum term.  The
// reference's cell-level pre-trim (NeighbourManager.h:367-474) only removes candidates
// this test rejects anyway, so it is not repeated.
#include "gsph_state.cuh"
#include "gsph_walk.cuh"
#include "kernels.cuh"

namespace gsph {

namespace {

constexpr int kForceWarps = 4;
constexpr int kForceStack = 1024;
constexpr int kForceList = 512;

template <int LPG>
__device__ __forceinline__ double gsum(double v) {
#pragma unroll
  for (int o = 1; o < LPG; o <<= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}

// GhostNeighbourFinder::PeriodicBoxOverlap (src/Headers/GhostNeighbours.hpp:202-226)
__device__ __forceinline__ bool periodic_box_overlap(const SphParams& prm, const double* amin,
                                                     const double* amax, const double* bmin,
                                                     const double* bmax) {
  if (!prm.periodic) return box_overlap(amin, amax, bmin, bmax);
  double corr[3];
  bool any = false;
  for (int k = 0; k < 3; k++) {
    const double dr = __dmul_rn(0.5, __dsub_rn(__dadd_rn(bmax[k], bmin[k]), __dadd_rn(amax[k], amin[k])));
    if (dr > prm.boxhalf[k]) { corr[k] = -prm.boxsize[k]; any = true; }
    else if (dr < -prm.boxhalf[k]) { corr[k] = prm.boxsize[k]; any = true; }
    else corr[k] = 0.0;
  }
  if (!any) return box_overlap(amin, amax, bmin, bmax);
  double pmin[3], pmax[3];
  for (int k = 0; k < 3; k++) { pmin[k] = __dadd_rn(bmin[k], corr[k]); pmax[k] = __dadd_rn(bmax[k], corr[k]); }
  return box_overlap(amin, amax, pmin, pmax);
}

// Per-lane accumulators of one particle.
struct Acc {
  double ah[3], ag[3], gpot, dudt, divv;
};

// Target particle data held by every lane of its group.
struct Target {
  double x, y, z, vx, vy, vz, m, h, invh, rho, invrho, hfactor, hrangesqd, fac, sound, zeta;
};

__device__ __forceinline__ void load_target(const Particles& p, int s, Target& T) {
  T.x = p.x[s]; T.y = p.y[s]; T.z = p.z[s];
  T.vx = p.vx[s]; T.vy = p.vy[s]; T.vz = p.vz[s];
  T.m = p.m[s]; T.h = p.h[s]; T.invh = 1.0 / T.h;
  T.rho = p.rho[s]; T.invrho = 1.0 / T.rho;
  T.hfactor = p.hfactor[s]; T.hrangesqd = p.hrangesqd[s];
  T.fac = (p.pressure[s] * p.invomega[s]) / (T.rho * T.rho);
  T.sound = p.sound[s]; T.zeta = p.zeta[s];
}

// Monaghan (1997) viscosity + grad-h pressure terms shared by both pair functions.
__device__ __forceinline__ double pair_pressure(const SphParams& prm, const Target& T, double wi, double wj,
                                                double facj, double invrhoj, double soundj, double mj,
                                                double dvdr, double& dudt) {
  double paux = T.fac * wi + facj * wj;
  if (dvdr < 0.0) {
    const double winvrho = 0.25 * (wi + wj) * (T.invrho + invrhoj);
    const double vsignal = T.sound + soundj - prm.beta_visc * prm.alpha_visc * dvdr;
    paux -= prm.alpha_visc * vsignal * dvdr * winvrho;
    dudt -= 0.5 * mj * prm.alpha_visc * vsignal * dvdr * dvdr * winvrho;
  }
  return paux;
}

// GradhSph::ComputeSphHydroForces, one pair (src/GradhSph/GradhSph.cpp:384-447).
__device__ __forceinline__ void hydro_pair(const SphParams& prm, const Particles& p, const Target& T, int j,
                                           double dx, double dy, double dz, double drsqd, Acc& A) {
  // the neighbour's quotients, computed once per particle (the same IEEE results as here)
  const double hj = p.h[j];
  const double invhj = p.invh_p[j], invrhoj = p.invrho_p[j];
  const double facj = p.fac_p[j];
  const double drmag = sqrt(drsqd);
  double ux = dx, uy = dy, uz = dz;
  if (drmag > 0.0) { const double inv = 1.0 / drmag; ux *= inv; uy *= inv; uz *= inv; }
  const double wi = T.hfactor * m4_w1(drmag * T.invh);
  const double wj = p.hfactor[j] * m4_w1(drmag * invhj);
  double dvdr = p.vx[j] * ux + p.vy[j] * uy + p.vz[j] * uz;
  dvdr -= T.vx * ux + T.vy * uy + T.vz * uz;
  const double mj = p.m[j];
  A.divv -= mj * dvdr * wi;
  const double paux = pair_pressure(prm, T, wi, wj, facj, invrhoj, p.sound[j], mj, dvdr, A.dudt);
  A.ah[0] += mj * ux * paux; A.ah[1] += mj * uy * paux; A.ah[2] += mj * uz * paux;
}

// GradhSph::ComputeSphHydroGravForces, one pair (src/GradhSph/GradhSph.cpp:498-571).
__device__ __forceinline__ void hydro_grav_pair(const SphParams& prm, const Particles& p, const Target& T,
                                                int j, double dx, double dy, double dz, double drsqd, Acc& A) {
  // the neighbour's quotients, computed once per particle (the same IEEE results as here)
  const double hj = p.h[j];
  const double invhj = p.invh_p[j], invrhoj = p.invrho_p[j];
  const double facj = p.fac_p[j];
  const double drmag = sqrt(drsqd + kSmall);
  const double invdrmag = 1.0 / drmag;
  const double ux = dx * invdrmag, uy = dy * invdrmag, uz = dz * invdrmag;
  const double dvdr = (p.vx[j] - T.vx) * ux + (p.vy[j] - T.vy) * uy + (p.vz[j] - T.vz) * uz;
  const double si = drmag * T.invh, sj = drmag * invhj;
  const double wi = T.hfactor * m4_w1(si);
  const double wj = p.hfactor[j] * m4_w1(sj);
  const double mj = p.m[j];
  const double paux = pair_pressure(prm, T, wi, wj, facj, invrhoj, p.sound[j], mj, dvdr, A.dudt);
  A.ah[0] += mj * ux * paux; A.ah[1] += mj * uy * paux; A.ah[2] += mj * uz * paux;
  // 1/s = h / |r|
  const double isi = T.h * invdrmag, isj = hj * invdrmag;
  const double pg = 0.5 * (T.invh * T.invh * m4_wgrav_r(si, isi) + T.zeta * wi +
                           invhj * invhj * m4_wgrav_r(sj, isj) + p.zeta[j] * wj);
  A.ag[0] += mj * ux * pg; A.ag[1] += mj * uy * pg; A.ag[2] += mj * uz * pg;
  A.gpot += 0.5 * mj * (T.invh * m4_wpot_r(si, isi) + invhj * m4_wpot_r(sj, isj));
  A.divv -= mj * dvdr * wi;
}

// GradhSphBase::ComputeDirectGravForces, one term (src/GradhSph/GradhSph.cpp:671-686).
__device__ __forceinline__ void direct_term(double dx, double dy, double dz, double mj, Acc& A) {
  const double drsqd = dx * dx + dy * dy + dz * dz + kSmall;
  const double invdrmag = rsqrt(drsqd);
  const double invdr3 = invdrmag * invdrmag * invdrmag;
  A.ag[0] += mj * dx * invdr3; A.ag[1] += mj * dy * invdr3; A.ag[2] += mj * dz * invdr3;
  A.gpot += mj * invdrmag;
}

// ComputeQuadropole<3> (src/Headers/NeighbourSearch.h:423-449) or the monopole term (:349-377).
__device__ __forceinline__ void cell_term(const CellMoment& c, const Target& T, bool quad, Acc& A) {
  const double dx = T.x - c.r[0], dy = T.y - c.r[1], dz = T.z - c.r[2];
  const double drsqd = dx * dx + dy * dy + dz * dz + kSmall;
  const double invdrmag = rsqrt(drsqd);
  const double invdrsqd = invdrmag * invdrmag;
  const double mon = c.m * invdrsqd * invdrmag;
  A.ag[0] -= mon * dx; A.ag[1] -= mon * dy; A.ag[2] -= mon * dz;
  A.gpot += c.m * invdrmag;
  if (quad) {
    const double* q = c.q;
    const double invdr5 = invdrsqd * invdrsqd * invdrmag;
    const double qzz = -(q[0] + q[2]);
    const double qscalar = q[0] * dx * dx + q[2] * dy * dy + qzz * dz * dz +
                           2.0 * (q[1] * dx * dy + q[3] * dx * dz + q[4] * dy * dz);
    const double qfactor = 2.5 * qscalar * invdr5 * invdrsqd;
    A.ag[0] += (q[0] * dx + q[1] * dy + q[3] * dz) * invdr5 - qfactor * dx;
    A.ag[1] += (q[1] * dx + q[2] * dy + q[4] * dz) * invdr5 - qfactor * dy;
    A.ag[2] += (q[3] * dx + q[4] * dy + qzz * dz) * invdr5 - qfactor * dz;
    A.gpot += 0.5 * qscalar * invdr5;
  }
}

template <int LPG>
__device__ __forceinline__ void reduce_acc(Acc& A) {
  for (int k = 0; k < 3; k++) { A.ah[k] = gsum<LPG>(A.ah[k]); A.ag[k] = gsum<LPG>(A.ag[k]); }
  A.gpot = gsum<LPG>(A.gpot);
  A.dudt = gsum<LPG>(A.dudt);
  A.divv = gsum<LPG>(A.divv);
}

__device__ __forceinline__ void finish_particle(const SphParams& prm, const Particles& p, int s, const Target& T,
                                                Acc& A, bool grav) {
  const double divv = A.divv * T.invrho;
  const double P = (prm.gamma_eos - 1.0) * T.rho * p.u[s];
  const double dudt = A.dudt - P * divv * T.invrho * p.invomega[s];
  p.div_v[s] = divv;
  p.dudt[s] = dudt;
  p.ax[s] = A.ah[0] + A.ag[0];
  p.ay[s] = A.ah[1] + A.ag[1];
  p.az[s] = A.ah[2] + A.ag[2];
  p.agx[s] = A.ag[0]; p.agy[s] = A.ag[1]; p.agz[s] = A.ag[2];
  p.gpot[s] = grav ? A.gpot : 0.0;
}

__device__ __forceinline__ unsigned long long warp_total(unsigned long long v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}

// ---- hydro only ------------------------------------------------------------------------
template <int LPG>
__global__ void __launch_bounds__(kForceWarps * 32)
k_hydro_fp64(Tree t, Particles p, SphParams prm, DeviceCounters cnt) {
  __shared__ int s_stack[kForceWarps][kForceStack];
  __shared__ int s_list[kForceWarps][kForceList];
  const int wib = threadIdx.x >> 5;
  const int leaf = blockIdx.x * kForceWarps + wib;
  if (leaf >= t.nleaf) return;
  const int lane = threadIdx.x & 31;
  const int g = lane / LPG, sl = lane % LPG;
  const int c = t.leaf_cell[leaf];
  const int first = t.cell_first[c], ncell = t.cell_n[c];
  const bool mine = g < ncell && is_active(p, first + g);
  if (!__any_sync(kFull, mine)) return;   // no active particle in this leaf
  const int slot = first + (g < ncell ? g : 0);
  int lvn_own = 0;
  Target T;
  load_target(p, slot, T);
  const CellGeom G = t.geom[c];
  const CellBox bb = t.bb[c], hb = t.hbox[c];
  Acc A = {};
  unsigned long long npairs = 0;
  WarpLists L{s_list[wib], s_list[wib], s_list[wib], 0, 0, 0, kForceList};
  auto decide = [&](int node, int level) -> int {
    if (t.cell_n[node] == 0) return kSkip;
    const CellBox ob = t.bb[node], oh = t.hbox[node];
    if (!(periodic_box_overlap(prm, bb.bbmin, bb.bbmax, oh.bbmin, oh.bbmax) ||
          periodic_box_overlap(prm, hb.bbmin, hb.bbmax, ob.bbmin, ob.bbmax))) return kSkip;
    return level == t.ltot ? kEmitA : kOpen;
  };
  auto tag = [](int node, int) { return node; };
  auto consume = [&]() {
    if (!mine) return;
    for (int e = 0; e < L.na; e++) {
      const int node = L.a[e];
      const int f = t.cell_first[node], nn = t.cell_n[node];
      for (int q = sl; q < nn; q += LPG) {
        const int j = f + q;
        double r[3] = {p.x[j], p.y[j], p.z[j]};
        int sh[3] = {0, 0, 0};   // image of j, in box lengths
        if (prm.periodic) {
          // GhostNeighbourFinder::_MakePeriodicGhost: image nearest the leaf centre
          double d[3];
          bool any = false;
          for (int k = 0; k < 3; k++) {
            d[k] = __dsub_rn(r[k], G.rcell[k]);
            if (d[k] > prm.boxhalf[k]) { d[k] = __dsub_rn(d[k], prm.boxsize[k]); any = true; sh[k] = -1; }
            else if (d[k] < -prm.boxhalf[k]) { d[k] = __dadd_rn(d[k], prm.boxsize[k]); any = true; sh[k] = 1; }
          }
          if (any) for (int k = 0; k < 3; k++) r[k] = __dadd_rn(G.rcell[k], d[k]);
        }
        double dx = __dsub_rn(r[0], T.x), dy = __dsub_rn(r[1], T.y), dz = __dsub_rn(r[2], T.z);
        if (prm.periodic) {
          // GhostNeighbourFinder::ApplyPeriodicDistanceCorrection relative to the particle
          double* dd[3] = {&dx, &dy, &dz};
          for (int k = 0; k < 3; k++) {
            if (*dd[k] > prm.boxhalf[k]) { *dd[k] = __dsub_rn(*dd[k], prm.boxsize[k]); sh[k]--; }
            else if (*dd[k] < -prm.boxhalf[k]) { *dd[k] = __dadd_rn(*dd[k], prm.boxsize[k]); sh[k]++; }
          }
          if ((sh[0] | sh[1] | sh[2]) && !ghost_exists(prm, p, j, sh)) continue;
        }
        const double drsqd = dot3_rn(dx, dy, dz);
        if (drsqd >= T.hrangesqd && drsqd >= p.hrangesqd[j]) continue;
        hydro_pair(prm, p, T, j, dx, dy, dz, drsqd, A);
        lvn_pair(p, slot, j, lvn_own);
        npairs++;
        if (cnt.record) {
          const int k = atomicAdd(&cnt.rec_sph_cnt[slot], 1);
          if (k < cnt.rec_max) cnt.rec_sph_ids[(size_t) slot * cnt.rec_max + k] = j;
        }
      }
    }
  };
  const bool ok = warp_walk(0, t.ltot, t.cell_level, s_stack[wib], kForceStack, L, decide, tag, consume);
  consume();
  if (!ok && lane == 0) atomicOr(cnt.status, (unsigned) kStatusStackOverflow);
  reduce_acc<LPG>(A);
  const unsigned long long tot = warp_total(npairs);
  if (lane == 0) atomicAdd(cnt.hydro_pairs, tot);
  lvn_finish(p, slot, mine, lvn_own);
  if (mine && sl == 0) finish_particle(prm, p, slot, T, A, false);
}

// ---- hydro + self-gravity ----------------------------------------------------------------
template <int LPG>
__global__ void __launch_bounds__(kForceWarps * 32)
k_all_forces_fp64(Tree t, Particles p, SphParams prm, DeviceCounters cnt) {
  __shared__ int s_stack[kForceWarps][kForceStack];
  __shared__ int s_la[kForceWarps][kForceList];
  __shared__ int s_lb[kForceWarps][kForceList];
  __shared__ int s_lc[kForceWarps][kForceList];
  const int wib = threadIdx.x >> 5;
  const int leaf = blockIdx.x * kForceWarps + wib;
  if (leaf >= t.nleaf) return;
  const int lane = threadIdx.x & 31;
  const int g = lane / LPG, sl = lane % LPG;
  const int c = t.leaf_cell[leaf];
  const int first = t.cell_first[c], ncell = t.cell_n[c];
  const bool mine = g < ncell && is_active(p, first + g);
  if (!__any_sync(kFull, mine)) return;   // no active particle in this leaf
  const int slot = first + (g < ncell ? g : 0);
  int lvn_own = 0;
  Target T;
  load_target(p, slot, T);
  const CellGeom G = t.geom[c];
  const bool quad = prm.multipole == 1;
  const double hrangemax = __dmul_rn(kKernRange, G.hmax);
  Acc A = {};
  A.gpot = mine && sl == 0 ? (T.m / T.h) * m4_wpot(0.0) : 0.0;
  unsigned long long nsph = 0, ndir = 0, ncellp = 0;
  unsigned long long dhash = 0, chash = 0, ccount = 0;
  WarpLists L{s_la[wib], s_lb[wib], s_lc[wib], 0, 0, 0, kForceList};
  auto decide = [&](int node, int level) -> int {
    const CellGeom o = t.geom[node];
    const int on = t.cell_n[node];
    const double dx = __dsub_rn(o.rcell[0], G.rcell[0]);
    const double dy = __dsub_rn(o.rcell[1], G.rcell[1]);
    const double dz = __dsub_rn(o.rcell[2], G.rcell[2]);
    const double drsqd = dot3_rn(dx, dy, dz);
    const double t1 = sq_rn(__dadd_rn(__dadd_rn(o.rmax, G.rmax), hrangemax));
    const double t2 = sq_rn(__dadd_rn(__dadd_rn(G.rmax, o.rmax), __dmul_rn(kKernRange, o.hmax)));
    if (drsqd <= t1 || drsqd <= t2) {
      if (level < t.ltot) return kOpen;
      return on == 0 ? kSkip : kEmitA;
    }
    if (on == 0) return kSkip;
    if (!(drsqd < o.cdistsqd)) return (level == t.ltot && on == 1) ? kEmitB : kEmitC;
    return level < t.ltot ? kOpen : kEmitB;
  };
  auto tag = [](int node, int) { return node; };
  auto consume = [&]() {
    if (!mine) return;
    // near leaf cells: SPH pair or direct term per pair
    for (int e = 0; e < L.na; e++) {
      const int node = L.a[e];
      const int f = t.cell_first[node], nn = t.cell_n[node];
      for (int q = sl; q < nn; q += LPG) {
        const int j = f + q;
        const double dx = __dsub_rn(p.x[j], T.x), dy = __dsub_rn(p.y[j], T.y), dz = __dsub_rn(p.z[j], T.z);
        const double drsqd = dot3_rn(dx, dy, dz);
        if (drsqd >= T.hrangesqd && drsqd >= p.hrangesqd[j]) {
          direct_term(dx, dy, dz, p.m[j], A);
          ndir++;
          if (cnt.record) { dhash += mix64((unsigned long long) p.id[j]); rec_direct_id(cnt, slot, p.id[j]); }
        } else {
          hydro_grav_pair(prm, p, T, j, dx, dy, dz, drsqd, A);
          lvn_pair(p, slot, j, lvn_own);
          nsph++;
          if (cnt.record) {
            const int k = atomicAdd(&cnt.rec_sph_cnt[slot], 1);
            if (k < cnt.rec_max) cnt.rec_sph_ids[(size_t) slot * cnt.rec_max + k] = j;
          }
        }
      }
    }
    // opened leaf cells beyond the near zone: direct terms
    for (int e = 0; e < L.nb; e++) {
      const int node = L.b[e];
      const int f = t.cell_first[node], nn = t.cell_n[node];
      for (int q = sl; q < nn; q += LPG) {
        const int j = f + q;
        direct_term(p.x[j] - T.x, p.y[j] - T.y, p.z[j] - T.z, p.m[j], A);
        ndir++;
        if (cnt.record) { dhash += mix64((unsigned long long) p.id[j]); rec_direct_id(cnt, slot, p.id[j]); }
      }
    }
    // accepted cells: multipole terms
    for (int e = sl; e < L.nc; e += LPG) {
      cell_term(t.mom[L.c[e]], T, quad, A);
      ncellp++;
      if (cnt.record && g == 0) {
        chash += mix64((unsigned long long) L.c[e]);
        ccount++;
        rec_cell_id(cnt, leaf, L.c[e]);
      }
    }
  };
  const bool ok = warp_walk(0, t.ltot, t.cell_level, s_stack[wib], kForceStack, L, decide, tag, consume);
  consume();
  if (!ok && lane == 0) atomicOr(cnt.status, (unsigned) kStatusStackOverflow);
  reduce_acc<LPG>(A);
  const unsigned long long a1 = warp_total(nsph), a2 = warp_total(ndir), a3 = warp_total(ncellp);
  if (lane == 0) {
    atomicAdd(cnt.hydro_pairs, a1);
    atomicAdd(cnt.direct_pairs, a2);
    atomicAdd(cnt.cell_pairs, a3);
  }
  if (cnt.record) {
    unsigned long long dc = ndir, dh = dhash;
    for (int o = 1; o < LPG; o <<= 1) {
      dc += __shfl_xor_sync(kFull, dc, o);
      dh += __shfl_xor_sync(kFull, dh, o);
    }
    if (mine && sl == 0) { cnt.rec_dir_cnt[slot] = dc; cnt.rec_dir_hash[slot] = dh; }
    const unsigned long long cc = warp_total(ccount), ch = warp_total(chash);
    if (lane == 0) { cnt.rec_cell_cnt[leaf] = cc; cnt.rec_cell_hash[leaf] = ch; }
  }
  lvn_finish(p, slot, mine, lvn_own);
  if (mine && sl == 0) finish_particle(prm, p, slot, T, A, true);
}

}  // namespace

#define GSPH_DISPATCH_LPG(KERNEL, LPG, ...)                                          \
  switch (LPG) {                                                                     \
    case 32: KERNEL<32><<<blocks, kForceWarps * 32, 0, st>>>(__VA_ARGS__); break;    \
    case 16: KERNEL<16><<<blocks, kForceWarps * 32, 0, st>>>(__VA_ARGS__); break;    \
    case 8: KERNEL<8><<<blocks, kForceWarps * 32, 0, st>>>(__VA_ARGS__); break;      \
    case 4: KERNEL<4><<<blocks, kForceWarps * 32, 0, st>>>(__VA_ARGS__); break;      \
    case 2: KERNEL<2><<<blocks, kForceWarps * 32, 0, st>>>(__VA_ARGS__); break;      \
    default: KERNEL<1><<<blocks, kForceWarps * 32, 0, st>>>(__VA_ARGS__); break;     \
  }

namespace {

// Per-particle quotients every pair of the FP64 force pass needs from its neighbour
// (GradhSph.cpp:398-402, :509-515 evaluate them per pair).
__global__ void k_pair_quotients_fp64(Particles p) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < p.n; s += gridDim.x * blockDim.x) {
    const double rho = p.rho[s];
    p.invh_p[s] = 1.0 / p.h[s];
    p.invrho_p[s] = 1.0 / rho;
    p.fac_p[s] = (p.pressure[s] * p.invomega[s]) / (rho * rho);
  }
}

void launch_pair_quotients(const Particles& p, cudaStream_t st) {
  const int blocks = (p.n + 255) / 256 < 152 * 8 ? (p.n + 255) / 256 : 152 * 8;
  k_pair_quotients_fp64<<<blocks > 0 ? blocks : 1, 256, 0, st>>>(p);
}

}  // namespace

void launch_hydro_forces(const Tree& t, const Particles& p, const SphParams& prm, const DeviceCounters& cnt,
                         int lanes_per_particle, cudaStream_t st) {
  launch_pair_quotients(p, st);
  const int blocks = (t.nleaf + kForceWarps - 1) / kForceWarps;
  GSPH_DISPATCH_LPG(k_hydro_fp64, lanes_per_particle, t, p, prm, cnt)
}

void launch_all_forces(const Tree& t, const Particles& p, const SphParams& prm, const DeviceCounters& cnt,
                       int lanes_per_particle, cudaStream_t st) {
  launch_pair_quotients(p, st);
  const int blocks = (t.nleaf + kForceWarps - 1) / kForceWarps;
  GSPH_DISPATCH_LPG(k_all_forces_fp64, lanes_per_particle, t, p, prm, cnt)
}

}  // namespace gsph
