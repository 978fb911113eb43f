// ORACLE — test infrastructure, not product code.
//
// CPU restatement of GANDALF's grad-h SPH + KD-tree gravity step, used only by tests/,
// __graft_entry__.smoke() and bench.py's CPU-baseline leg as the checker.  It follows the
// reference algorithm step by step (citations are to the GANDALF source tree):
//
//   tree build   KDTree::BuildTree / DivideTreeCell / QuickSelect   src/Tree/KDTree.cpp:219-750
//   stock        KDTree::StockCellProperties                         src/Tree/KDTree.cpp:807-1083
//   h-rho solve  GradhSphTree::UpdateAllSphProperties                src/GradhSph/GradhSphTree.cpp:82-271
//                Tree::ComputeGatherNeighbourList                    src/Tree/Tree.cpp:290-381
//                GradhSph::ComputeH                                  src/GradhSph/GradhSph.cpp:141-326
//   hmax update  KDTree::UpdateHmaxValues                            src/Tree/KDTree.cpp:1127-1208
//   hydro        GradhSphTree::UpdateAllSphHydroForces               src/GradhSph/GradhSphTree.cpp:279-435
//                Tree::ComputeNeighbourAndGhostList                  src/Tree/Tree.cpp:561-617
//                NeighbourManager::_EndSearch / TrimNeighbourLists   src/Headers/NeighbourManager.h:367-543
//                GradhSph::ComputeSphHydroForces                     src/GradhSph/GradhSph.cpp:360-460
//   gravity      GradhSphTree::UpdateAllSphForces                    src/GradhSph/GradhSphTree.cpp:443-657
//                Tree::ComputeGravityInteractionAndGhostList         src/Tree/Tree.cpp:627-735
//                GradhSph::ComputeSphHydroGravForces                 src/GradhSph/GradhSph.cpp:473-585
//                GradhSphBase::ComputeDirectGravForces               src/GradhSph/GradhSph.cpp:656-690
//                ComputeQuadropole<3> / ComputeCellQuadrupoleForces  src/Headers/NeighbourSearch.h:423-475
//   kernel       M4Kernel (analytic, 3-D norm 1/pi)                  src/Headers/SmoothingKernel.h:131-240
//
// Periodic images for the density gather follow the reference's ghost particles
// (Hydrodynamics::CheckBoundaryGhostParticle, src/Hydrodynamics/Hydrodynamics.cpp:217-247):
// an image r +- L of particle j exists in dimension k when r_k lies within
// ghost_range*kernrange*h_j = 5 h_j of the boundary, h_j taken before the h solve.
// Hydro-force images follow GhostNeighbourFinder::_MakePeriodicGhost (nearest image of
// the particle relative to the leaf-cell centre, src/Headers/GhostNeighbours.hpp:349-362).
//
// Build with -ffp-contract=off so that x86-64 and aarch64 give the same bits.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

const double kInvPi = 0.31830988618379;   // reference constant, src/Headers/Constants.h:63
const double kSmall = 1.0e-20;            // src/Headers/Constants.h:73
const double kBig = 9.9e20;               // src/Headers/Constants.h:72
const double kKernRange = 2.0;
const double kKernRangeSqd = 4.0;
const double kGhostRange = 2.5;           // src/Headers/Hydrodynamics.h:52
const double kTwoPi = 6.28318530717959;   // src/Headers/Constants.h:62

struct Params {
  int32_t self_gravity, eos, periodic, nleafmax, multipole, hydro_forces, pad0, pad1;
  double h_fac, h_converge, alpha_visc, beta_visc, gamma_eos, thetamaxsqd, temp0, mu_bar;
  double boxmin[3], boxmax[3];
};

// ---- M4 kernel (SmoothingKernel.h:131-240) --------------------------------------------
inline double w0(double s) {
  if (s < 1.0) return kInvPi * (1.0 - 1.5 * s * s + 0.75 * s * s * s);
  if (s < 2.0) return 0.25 * kInvPi * std::pow(2.0 - s, 3);
  return 0.0;
}
inline double w1(double s) {
  if (s < 1.0) return kInvPi * (-3.0 * s + 2.25 * s * s);
  if (s < 2.0) return -0.75 * kInvPi * (2.0 - s) * (2.0 - s);
  return 0.0;
}
inline double womega(double s) {
  const double nd = 3.0;
  if (s < 1.0) return kInvPi * (-nd + 1.5 * (nd + 2.0) * s * s - 0.75 * (nd + 3.0) * std::pow(s, 3));
  if (s < 2.0)
    return kInvPi * (-2.0 * nd + 3.0 * (nd + 1.0) * s - 1.50 * (nd + 2.0) * s * s +
                     0.25 * (nd + 3.0) * std::pow(s, 3));
  return 0.0;
}
inline double wzeta(double s) {
  if (s < 1.0) return 1.4 - 2.0 * s * s + 1.5 * std::pow(s, 4) - 0.6 * std::pow(s, 5);
  if (s < 2.0)
    return 1.6 - 4.0 * s * s + 4.0 * std::pow(s, 3) - 1.5 * std::pow(s, 4) + 0.2 * std::pow(s, 5);
  return 0.0;
}
inline double wgrav(double s) {
  if (s < 1.0) return 1.333333333333333333333 * s - 1.2 * std::pow(s, 3) + 0.5 * std::pow(s, 4);
  if (s < 2.0)
    return 2.6666666666666666667 * s - 3.0 * s * s + 1.2 * std::pow(s, 3) -
           0.166666666666666666667 * std::pow(s, 4) - 0.06666666666666666667 / (s * s);
  return 1.0 / (s * s);
}
inline double wpot(double s) {
  if (s < 1.0) return 1.4 - 0.666666666666666666666666 * s * s + 0.3 * std::pow(s, 4) - 0.1 * std::pow(s, 5);
  if (s < 2.0)
    return -1.0 / (15.0 * s) + 1.6 - 1.33333333333333333333333333 * s * s + std::pow(s, 3) -
           0.3 * std::pow(s, 4) + (1.0 / 30.0) * std::pow(s, 5);
  return 1.0 / s;
}

inline double dot3(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

// splitmix64 term summed per list entry: an order-independent list hash.
inline uint64_t mix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

struct Cell {
  int n, level, first;             // particles [first, first+n) of the leaf-ordered arrays
  double bbmin[3], bbmax[3], hbmin[3], hbmax[3], rcell[3], r[3], q[5];
  double m, rmax, hmax, cdistsqd, maxsound;
};

struct Oracle {
  Params p;
  int64_t n = 0;
  int ltot = 0, ncell = 0;
  // particle data in input order
  std::vector<double> x[3], v[3], m, u, h, h_ghost;
  // leaf order: order[pos] = particle id
  std::vector<int> order;
  std::vector<Cell> cells;
  std::vector<int> leaves;         // DFS ids of leaves, left to right
  // outputs (input order)
  std::vector<double> rho, invomega, zeta, hfactor, pressure, sound, div_v, dudt, gpot, hrangesqd;
  std::vector<double> a[3], ag[3], gpot_hydro;
  // star particles (NbodyParticle r, v, m, h) and the star <- gas results
  int nstar = 0;
  std::vector<double> sx[3], sv[3], sm, sh;
  std::vector<double> s_a[3], s_adot[3], s_gpot;
  // optional lists
  bool want_lists = false;
  std::vector<std::vector<int>> hydro_neib, direct_neib;   // per particle (input ids)
  std::vector<std::vector<int>> gcell_list;                // per leaf (DFS ids)
  std::vector<int> gcell_leaf;
  bool want_summary = false;                               // (count, hash) instead of lists
  std::vector<int64_t> dir_count, cell_count;
  std::vector<uint64_t> dir_hash, cell_hash;
  int64_t n_density_pairs = 0, n_hydro_pairs = 0, n_direct_pairs = 0, n_cell_pairs = 0;
  // Active particles (the reference's `active` flag, src/Headers/Flags.h:33): empty means
  // every particle is active.  The h solve and the force passes work on active particles
  // only (Tree::ComputeActiveCellList / ComputeActiveParticleList, src/Tree/Tree.cpp:59-115).
  std::vector<unsigned char> active;
  // Timestep levels, and the neighbour-level bookkeeping of a force pass
  // (GradhSph.cpp:445-446, :569-570; GradhSphTree.cpp:375-417, :610-640).  Empty: not kept.
  std::vector<int> level, levelneib;
  bool is_active(int64_t i) const { return active.empty() || active[i]; }
  bool leaf_has_active(const Cell& cell) const {
    if (active.empty()) return cell.n > 0;
    for (int j = 0; j < cell.n; j++)
      if (active[order[cell.first + j]]) return true;
    return false;
  }

  int c2_of(int c, int level) const { return c + (1 << (ltot - level)); }
  int cnext_of(int c, int level) const {
    return level == ltot ? c + 1 : c + (1 << (ltot - level + 1)) - 1;
  }

  // ---------------------------------------------------------------------------------
  // KD-tree build: same topology, boxes and median splits as KDTree::BuildTree.
  // Ties at a median are broken by particle id (the reference breaks them by QuickSelect
  // order; the two agree whenever coordinates are distinct).
  void build_tree() {
    ltot = 0;
    while ((double) p.nleafmax * std::pow(2.0, ltot) < (double) n) ltot++;
    ncell = 2 * (1 << ltot) - 1;
    cells.assign(ncell, Cell());
    order.resize(n);
    std::iota(order.begin(), order.end(), 0);
    double bmin[3], bmax[3];
    for (int k = 0; k < 3; k++) { bmin[k] = kBig; bmax[k] = -kBig; }
    for (int64_t i = 0; i < n; i++)
      for (int k = 0; k < 3; k++) {
        bmax[k] = std::max(bmax[k], x[k][i] + kKernRange * h[i]);
        bmin[k] = std::min(bmin[k], x[k][i] - kKernRange * h[i]);
      }
    leaves.clear();
    divide(0, 0, 0, (int) n, bmin, bmax);
  }

  void divide(int c, int level, int first, int cnt, const double* bbmin, const double* bbmax) {
    Cell& cell = cells[c];
    cell.level = level; cell.first = first; cell.n = cnt;
    if (level == ltot) { leaves.push_back(c); stock_leaf(c); return; }
    int kd = 0; double rkmax = 0.0;
    for (int k = 0; k < 3; k++)
      if (bbmax[k] - bbmin[k] > rkmax) { rkmax = bbmax[k] - bbmin[k]; kd = k; }
    const int half = cnt / 2;
    double rdivide = 0.0;
    if (cnt > 0) {
      const std::vector<double>& xk = x[kd];
      std::nth_element(order.begin() + first, order.begin() + first + half, order.begin() + first + cnt,
                       [&](int a_, int b_) { return xk[a_] < xk[b_] || (xk[a_] == xk[b_] && a_ < b_); });
      rdivide = xk[order[first + half]];
    }
    double b1max[3], b2min[3];
    std::memcpy(b1max, bbmax, sizeof(b1max)); b1max[kd] = rdivide;
    std::memcpy(b2min, bbmin, sizeof(b2min)); b2min[kd] = rdivide;
    divide(c + 1, level + 1, first, half, bbmin, b1max);
    divide(c2_of(c, level), level + 1, first + half, cnt - half, b2min, bbmax);
    stock_parent(c);
  }

  void finish_geometry(Cell& cell) {
    if (cell.n > 0) {
      double dr[3];
      for (int k = 0; k < 3; k++) cell.rcell[k] = 0.5 * (cell.bbmin[k] + cell.bbmax[k]);
      for (int k = 0; k < 3; k++) dr[k] = 0.5 * (cell.bbmax[k] - cell.bbmin[k]);
      cell.cdistsqd = std::max(dot3(dr, dr), cell.hmax * cell.hmax) / p.thetamaxsqd;
      cell.rmax = std::sqrt(dot3(dr, dr));
    }
  }

  void stock_leaf(int c) {
    Cell& cell = cells[c];
    cell.m = 0; cell.hmax = 0; cell.rmax = 0; cell.cdistsqd = kBig; cell.maxsound = 0;
    for (int k = 0; k < 5; k++) cell.q[k] = 0;
    for (int k = 0; k < 3; k++) {
      cell.r[k] = 0; cell.rcell[k] = 0;
      cell.bbmin[k] = kBig; cell.bbmax[k] = -kBig; cell.hbmin[k] = kBig; cell.hbmax[k] = -kBig;
    }
    for (int j = 0; j < cell.n; j++) {
      const int i = order[cell.first + j];
      cell.hmax = std::max(cell.hmax, h[i]);
      cell.m += m[i];
      for (int k = 0; k < 3; k++) cell.r[k] += m[i] * x[k][i];
      for (int k = 0; k < 3; k++) {
        if (x[k][i] < cell.bbmin[k]) cell.bbmin[k] = x[k][i];
        if (x[k][i] > cell.bbmax[k]) cell.bbmax[k] = x[k][i];
        if (x[k][i] - kKernRange * h[i] < cell.hbmin[k]) cell.hbmin[k] = x[k][i] - kKernRange * h[i];
        if (x[k][i] + kKernRange * h[i] > cell.hbmax[k]) cell.hbmax[k] = x[k][i] + kKernRange * h[i];
      }
    }
    if (cell.m > 0) for (int k = 0; k < 3; k++) cell.r[k] /= cell.m;
    finish_geometry(cell);
    for (int j = 0; j < cell.n; j++) {
      const int i = order[cell.first + j];
      double dr[3];
      for (int k = 0; k < 3; k++) dr[k] = x[k][i] - cell.r[k];
      const double drsqd = dot3(dr, dr);
      cell.q[0] += m[i] * (3.0 * dr[0] * dr[0] - drsqd);
      cell.q[1] += m[i] * 3.0 * dr[0] * dr[1];
      cell.q[2] += m[i] * (3.0 * dr[1] * dr[1] - drsqd);
      cell.q[3] += m[i] * 3.0 * dr[2] * dr[0];
      cell.q[4] += m[i] * 3.0 * dr[2] * dr[1];
    }
  }

  void stock_parent(int c) {
    Cell& cell = cells[c];
    const Cell& c1 = cells[c + 1];
    const Cell& c2 = cells[c2_of(c, cell.level)];
    cell.hmax = 0; cell.maxsound = 0; cell.cdistsqd = kBig; cell.rmax = 0;
    for (int k = 0; k < 5; k++) cell.q[k] = 0;
    for (int k = 0; k < 3; k++) {
      cell.r[k] = 0; cell.rcell[k] = 0;
      cell.bbmin[k] = kBig; cell.bbmax[k] = -kBig; cell.hbmin[k] = kBig; cell.hbmax[k] = -kBig;
    }
    for (const Cell* ch : {&c1, &c2}) {
      if (ch->n <= 0) continue;
      for (int k = 0; k < 3; k++) {
        cell.bbmin[k] = std::min(ch->bbmin[k], cell.bbmin[k]);
        cell.bbmax[k] = std::max(ch->bbmax[k], cell.bbmax[k]);
        cell.hbmin[k] = std::min(ch->hbmin[k], cell.hbmin[k]);
        cell.hbmax[k] = std::max(ch->hbmax[k], cell.hbmax[k]);
      }
      cell.hmax = std::max(cell.hmax, ch->hmax);
    }
    cell.n = c1.n + c2.n;
    cell.m = c1.m + c2.m;
    if (cell.m > 0)
      for (int k = 0; k < 3; k++) cell.r[k] = (c1.m * c1.r[k] + c2.m * c2.r[k]) / cell.m;
    finish_geometry(cell);
    for (const Cell* ch : {&c1, &c2}) {
      if (!(ch->m > 0)) continue;
      double dr[3];
      for (int k = 0; k < 3; k++) dr[k] = ch->r[k] - cell.r[k];
      const double drsqd = dot3(dr, dr);
      for (int k = 0; k < 5; k++) cell.q[k] += ch->q[k];
      cell.q[0] += ch->m * (3.0 * dr[0] * dr[0] - drsqd);
      cell.q[1] += ch->m * 3.0 * dr[0] * dr[1];
      cell.q[2] += ch->m * (3.0 * dr[1] * dr[1] - drsqd);
      cell.q[3] += ch->m * 3.0 * dr[2] * dr[0];
      cell.q[4] += ch->m * 3.0 * dr[2] * dr[1];
    }
  }

  // KDTree::UpdateHmaxValues: hmax and hbox from the solved h (cdistsqd untouched).
  void update_hmax(int c) {
    Cell& cell = cells[c];
    if (cell.level != ltot) { update_hmax(c + 1); update_hmax(c2_of(c, cell.level)); }
    cell.hmax = 0;
    for (int k = 0; k < 3; k++) { cell.hbmin[k] = kBig; cell.hbmax[k] = -kBig; }
    if (cell.level == ltot) {
      for (int j = 0; j < cell.n; j++) {
        const int i = order[cell.first + j];
        cell.hmax = std::max(cell.hmax, h[i]);
        for (int k = 0; k < 3; k++) {
          if (x[k][i] - kKernRange * h[i] < cell.hbmin[k]) cell.hbmin[k] = x[k][i] - kKernRange * h[i];
          if (x[k][i] + kKernRange * h[i] > cell.hbmax[k]) cell.hbmax[k] = x[k][i] + kKernRange * h[i];
        }
      }
    } else {
      for (int cc : {c + 1, c2_of(c, cell.level)}) {
        const Cell& ch = cells[cc];
        if (ch.n <= 0) continue;
        cell.hmax = std::max(cell.hmax, ch.hmax);
        for (int k = 0; k < 3; k++) {
          cell.hbmin[k] = std::min(ch.hbmin[k], cell.hbmin[k]);
          cell.hbmax[k] = std::max(ch.hbmax[k], cell.hbmax[k]);
        }
      }
    }
  }

  static bool box_overlap(const double* amin, const double* amax, const double* bmin, const double* bmax) {
    for (int k = 0; k < 3; k++) {
      if (amin[k] > bmax[k]) return false;
      if (bmin[k] > amax[k]) return false;
    }
    return true;
  }

  // Stackless walk: visit(cell) returns true to open (descend) the cell.
  template <class F>
  void walk(F visit) const {
    int c = 0;
    while (c < ncell) {
      const Cell& cell = cells[c];
      const int act = visit(c, cell);   // 0 skip, 1 open
      if (act == 1 && cell.level < ltot) c = c + 1;
      else c = cnext_of(c, cell.level);
    }
  }

  double eos_pressure(double rho_, double u_) const { return (p.gamma_eos - 1.0) * rho_ * u_; }

  // ---------------------------------------------------------------------------------
  // h-rho solve for one particle (GradhSph::ComputeH).  Returns 0 when h exceeds hmax.
  struct Ngb { double r[3]; double m; };
  int compute_h(int i, double hmax, const std::vector<Ngb>& ngbs, int64_t& pairs) {
    int iteration = 0;
    const int iteration_max = 30;
    double h_lower = 0.0, h_upper = hmax;
    double hi = h[i];
    double rho_ = 0, invom = 0, zet = 0, hfac = 0, invh = 0, invhsqd = 0;
    const double mi = m[i];
    const double rp[3] = {x[0][i], x[1][i], x[2][i]};
    const double invndim = 1.0 / 3.0;
    auto h_rho = [&](double rr) { return p.h_fac * std::pow(mi / rr, invndim); };
    do {
      iteration++;
      invh = 1.0 / hi;
      rho_ = 0; invom = 0; zet = 0;
      hfac = std::pow(invh, 3);
      invhsqd = invh * invh;
      for (const Ngb& g : ngbs) {
        double dr[3];
        for (int k = 0; k < 3; k++) dr[k] = g.r[k] - rp[k];
        const double ssqd = invhsqd * dot3(dr, dr);
        const double s = std::sqrt(ssqd);
        rho_ += g.m * w0(s);
        invom += g.m * invh * womega(s);
        zet += g.m * wzeta(s);
      }
      pairs += (int64_t) ngbs.size();
      rho_ *= hfac; invom *= hfac; zet *= invhsqd;
      if (rho_ > 0.0 && hi > h_lower && std::fabs(hi - h_rho(rho_)) * invh < p.h_converge) break;
      if (iteration < iteration_max) hi = h_rho(rho_);
      else if (iteration == iteration_max) hi = 0.5 * (h_lower + h_upper);
      else if (iteration < 5 * iteration_max) {
        if (rho_ < kSmall || hi > h_rho(rho_)) h_upper = hi; else h_lower = hi;
        hi = 0.5 * (h_lower + h_upper);
      } else {
        return -2;   // the reference raises "Problem with convergence of h-rho iteration"
      }
      if (hi > hmax) return 0;
    } while (hi > h_lower && hi < h_upper);
    hi = std::max(h_rho(rho_), h_lower);
    invh = 1.0 / hi;
    h[i] = hi;
    rho[i] = rho_;
    hfactor[i] = std::pow(invh, 3 + 1);
    hrangesqd[i] = kKernRangeSqd * hi * hi;
    div_v[i] = 0.0;
    const double drho = -invndim * hi / rho_;   // Sph.h:264-268
    invom = 1.0 - drho * invom;
    invomega[i] = 1.0 / invom;
    // SPH-star conservative-gravity zeta term (Hubber et al. 2013; GradhSph.cpp:282-297,
    // the default conservative_sph_star_gravity = 1 with softened N-body gravity)
    for (int s_ = 0; s_ < nstar; s_++) {
      const double ih = 2.0 / (hi + sh[s_]);
      const double ihsqd = ih * ih;
      double dr[3];
      for (int k = 0; k < 3; k++) dr[k] = sx[k][s_] - rp[k];
      const double ssqd = dot3(dr, dr) * ihsqd;
      zet += sm[s_] * ihsqd * wzeta(std::sqrt(ssqd));
    }
    zeta[i] = drho * zet * invomega[i];
    // thermal properties (GradhSph::ComputeThermalProperties, EOS)
    if (p.eos == 1) u[i] = p.temp0 / (p.gamma_eos - 1.0) / p.mu_bar;
    sound[i] = p.eos == 1 ? std::sqrt((p.gamma_eos - 1.0) * u[i])
                          : std::sqrt(p.gamma_eos * (p.gamma_eos - 1.0) * u[i]);
    pressure[i] = eos_pressure(rho[i], u[i]);
    return 1;
  }

  // Periodic shifts a gather box needs (one list per dimension), with ghost semantics.
  void gather_for_leaf(int c, double hmax, std::vector<Ngb>& out) {
    const Cell& cell = cells[c];
    out.clear();
    double gmin[3], gmax[3];
    for (int k = 0; k < 3; k++) { gmin[k] = cell.bbmin[k] - kKernRange * hmax; gmax[k] = cell.bbmax[k] + kKernRange * hmax; }
    const double hrangemaxsqd = std::pow(cell.rmax + kKernRange * hmax, 2);
    int ns[3] = {1, 1, 1};
    double sh[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    if (p.periodic) {
      for (int k = 0; k < 3; k++) {
        const double L = p.boxmax[k] - p.boxmin[k];
        // real particles near the far side appear as ghosts at r +- L
        if (gmax[k] > p.boxmax[k]) sh[k][ns[k]++] = L;    // ghosts of lhs particles (r + L)
        if (gmin[k] < p.boxmin[k]) sh[k][ns[k]++] = -L;   // ghosts of rhs particles (r - L)
      }
    }
    for (int a0 = 0; a0 < ns[0]; a0++)
      for (int a1 = 0; a1 < ns[1]; a1++)
        for (int a2 = 0; a2 < ns[2]; a2++) {
          const double s[3] = {sh[0][a0], sh[1][a1], sh[2][a2]};
          double bmin[3], bmax[3];
          for (int k = 0; k < 3; k++) { bmin[k] = gmin[k] - s[k]; bmax[k] = gmax[k] - s[k]; }
          walk([&](int cc, const Cell& o) -> int {
            if (!box_overlap(bmin, bmax, o.bbmin, o.bbmax)) return 0;
            if (o.level < ltot) return 1;
            for (int j = 0; j < o.n; j++) {
              const int id = order[o.first + j];
              Ngb g;
              bool ok = true;
              for (int k = 0; k < 3; k++) {
                if (s[k] == 0.0) { g.r[k] = x[k][id]; continue; }
                const double lim = kGhostRange * kKernRange * h_ghost[id];
                if (s[k] > 0.0) ok = ok && (x[k][id] < p.boxmin[k] + lim);
                else ok = ok && (x[k][id] > p.boxmax[k] - lim);
                g.r[k] = x[k][id] + s[k];
              }
              if (!ok) continue;
              double dr[3];
              for (int k = 0; k < 3; k++) dr[k] = g.r[k] - cell.rcell[k];
              if (dot3(dr, dr) < hrangemaxsqd) { g.m = m[id]; out.push_back(g); }
            }
            return 0;
          });
        }
  }

  int density() {
    int status = 0;
#pragma omp parallel
    {
      std::vector<Ngb> cand, ngb2;
      int64_t local_pairs = 0;
#pragma omp for schedule(guided)
      for (int li = 0; li < (int) leaves.size(); li++) {
        const int c = leaves[li];
        const Cell& cell = cells[c];
        if (!leaf_has_active(cell)) continue;
        double hmax = cell.hmax;
        std::vector<double> hsave(cell.n);
        for (int j = 0; j < cell.n; j++) hsave[j] = h[order[cell.first + j]];
        bool done;
        do {
          hmax = 1.05 * hmax;
          done = true;
          for (int j = 0; j < cell.n; j++) h[order[cell.first + j]] = hsave[j];
          gather_for_leaf(c, hmax, cand);
          for (int j = 0; j < cell.n; j++) {
            const int i = order[cell.first + j];
            if (!is_active(i)) continue;
            const double rp[3] = {x[0][i], x[1][i], x[2][i]};
            const double hrs = kKernRangeSqd * hmax * hmax;
            ngb2.clear();
            for (const Ngb& g : cand) {
              double dr[3];
              for (int k = 0; k < 3; k++) dr[k] = g.r[k] - rp[k];
              if (dot3(dr, dr) + kSmall <= hrs) ngb2.push_back(g);
            }
            const int ok = compute_h(i, hmax, ngb2, local_pairs);
            if (ok == -2) {
#pragma omp atomic write
              status = -2;
            }
            if (ok == 0) { done = false; break; }
          }
        } while (!done);
      }
#pragma omp atomic
      n_density_pairs += local_pairs;
    }
    return status;
  }

  // ---------------------------------------------------------------------------------
  // Hydro-only forces (periodic or open) for all particles.
  void hydro_forces() {
    begin_levels();
#pragma omp parallel
    {
      std::vector<int> cand_id;
      std::vector<double> cand_r;
      int64_t local_pairs = 0;
      int* lv = thread_levels();
#pragma omp for schedule(guided)
      for (int li = 0; li < (int) leaves.size(); li++) {
        const Cell& cell = cells[leaves[li]];
        if (!leaf_has_active(cell)) continue;
        cand_id.clear(); cand_r.clear();
        const double hrangemaxsqd = std::pow(cell.rmax + kKernRange * cell.hmax, 2);
        walk([&](int cc, const Cell& o) -> int {
          if (!(periodic_box_overlap(cell.bbmin, cell.bbmax, o.hbmin, o.hbmax) ||
                periodic_box_overlap(cell.hbmin, cell.hbmax, o.bbmin, o.bbmax))) return 0;
          if (o.level < ltot) return 1;
          for (int j = 0; j < o.n; j++) {
            const int id = order[o.first + j];
            double r[3] = {x[0][id], x[1][id], x[2][id]};
            nearest_image_about(cell.rcell, r);
            double dr[3];
            for (int k = 0; k < 3; k++) dr[k] = r[k] - cell.rcell[k];
            const double drsqd = dot3(dr, dr);
            const double h2 = cell.rmax + kKernRange * h[id];
            if (drsqd < hrangemaxsqd || drsqd < h2 * h2) {
              cand_id.push_back(id);
              for (int k = 0; k < 3; k++) cand_r.push_back(r[k]);
            }
          }
          return 0;
        });
        for (int j = 0; j < cell.n; j++) {
          const int i = order[cell.first + j];
          if (!is_active(i)) continue;
          pair_loop(i, cand_id, cand_r, false, nullptr, local_pairs, lv);
        }
      }
#pragma omp atomic
      n_hydro_pairs += local_pairs;
    }
    end_levels();
  }

  // Per-thread neighbour-level buffers (the reference's levelneibbuf, HydroTree.cpp:230-240)
  // and their reduction into levelneib: an active particle's levelneib restarts from 0
  // (Sph::ZeroAccelerations, src/Hydrodynamics/Sph.cpp:126-140) and every particle takes
  // the max with what the pass found (GradhSphTree.cpp:412-417, :635-640).
  std::vector<std::vector<int>> lvbuf;
  void begin_levels() {
    if (level.empty()) return;
    int nt = 1;
#ifdef _OPENMP
    nt = omp_get_max_threads();
#endif
    lvbuf.assign(nt, std::vector<int>(n, 0));
  }
  int* thread_levels() {
    if (level.empty()) return nullptr;
    int t = 0;
#ifdef _OPENMP
    t = omp_get_thread_num();
#endif
    return lvbuf[t].data();
  }
  void end_levels() {
    if (level.empty()) return;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) {
      int v = is_active(i) ? 0 : levelneib[i];
      for (const auto& b : lvbuf) v = std::max(v, b[i]);
      levelneib[i] = v;
    }
    lvbuf.clear();
  }

  bool periodic_box_overlap(const double* amin, const double* amax, const double* bmin, const double* bmax) const {
    if (!p.periodic) return box_overlap(amin, amax, bmin, bmax);
    double dr[3], corr[3];
    bool any = false;
    for (int k = 0; k < 3; k++) dr[k] = 0.5 * ((bmax[k] + bmin[k]) - (amax[k] + amin[k]));
    for (int k = 0; k < 3; k++) {
      const double L = p.boxmax[k] - p.boxmin[k], half = 0.5 * L;
      if (dr[k] > half) { corr[k] = -L; any = true; }
      else if (dr[k] < -half) { corr[k] = L; any = true; }
      else corr[k] = 0;
    }
    if (!any) return box_overlap(amin, amax, bmin, bmax);
    double pmin[3], pmax[3];
    for (int k = 0; k < 3; k++) { pmin[k] = bmin[k] + corr[k]; pmax[k] = bmax[k] + corr[k]; }
    return box_overlap(amin, amax, pmin, pmax);
  }

  // GhostNeighbourFinder::_MakePeriodicGhost: image of r nearest to centre.
  void nearest_image_about(const double* centre, double* r) const {
    if (!p.periodic) return;
    double dr[3];
    bool any = false;
    for (int k = 0; k < 3; k++) dr[k] = r[k] - centre[k];
    for (int k = 0; k < 3; k++) {
      const double L = p.boxmax[k] - p.boxmin[k], half = 0.5 * L;
      if (dr[k] > half) { dr[k] -= L; any = true; }
      else if (dr[k] < -half) { dr[k] += L; any = true; }
    }
    if (any) for (int k = 0; k < 3; k++) r[k] = centre[k] + dr[k];
  }

  // Pair loop over candidate SPH neighbours of particle i (hydro or hydro+gravity).
  // With gravity, candidates that fail the SPH test are Newtonian direct terms.
  void pair_loop(int i, const std::vector<int>& cid, const std::vector<double>& cr, bool grav,
                 std::vector<int>* direct_out, int64_t& pairs, int* lv = nullptr) {
    const double hi = h[i], rhoi = rho[i];
    const double invh_i = 1.0 / hi, invrho_i = 1.0 / rhoi, invhsqdi = invh_i * invh_i;
    const double rp[3] = {x[0][i], x[1][i], x[2][i]};
    const double vi[3] = {v[0][i], v[1][i], v[2][i]};
    const double fac_i = (pressure[i] * invomega[i]) / (rhoi * rhoi);
    double acc[3] = {0, 0, 0}, accg[3] = {0, 0, 0}, divv = 0, du = 0, pot = 0;
    std::vector<int> direct_local;
    for (size_t q = 0; q < cid.size(); q++) {
      const int j = cid[q];
      double rj[3] = {cr[3 * q], cr[3 * q + 1], cr[3 * q + 2]};
      double draux[3];
      for (int k = 0; k < 3; k++) draux[k] = rj[k] - rp[k];
      if (p.periodic) {
        for (int k = 0; k < 3; k++) {
          const double L = p.boxmax[k] - p.boxmin[k], half = 0.5 * L;
          if (draux[k] > half) { draux[k] += -L; rj[k] += -L; }
          else if (draux[k] < -half) { draux[k] += L; rj[k] += L; }
        }
      }
      const double drsqd = dot3(draux, draux);
      if (drsqd >= hrangesqd[i] && drsqd >= hrangesqd[j]) {
        if (grav) direct_local.push_back(q);
        continue;
      }
      if (want_lists || want_summary) hydro_neib[i].push_back(j);
      pairs++;
      if (lv) {   // GradhSph.cpp:445-446 / :569-570
        lv[i] = std::max(lv[i], level[j]);
        lv[j] = std::max(lv[j], level[i]);
      }
      const double invh_j = 1.0 / h[j], invrho_j = 1.0 / rho[j];
      const double fac_j = (pressure[j] * invomega[j]) / (rho[j] * rho[j]);
      if (!grav) {
        // GradhSph::ComputeSphHydroForces
        double dr[3] = {draux[0], draux[1], draux[2]};
        const double drmag = std::sqrt(dot3(dr, dr));
        if (drmag > 0) for (int k = 0; k < 3; k++) dr[k] /= drmag;
        const double wi = hfactor[i] * w1(drmag * invh_i);
        const double wj = hfactor[j] * w1(drmag * invh_j);
        const double vj[3] = {v[0][j], v[1][j], v[2][j]};
        double dvdr = dot3(vj, dr);
        dvdr -= dot3(vi, dr);
        divv -= m[j] * dvdr * wi;
        double paux = fac_i * wi + fac_j * wj;
        if (dvdr < 0.0) {
          const double winvrho = 0.25 * (wi + wj) * (invrho_i + invrho_j);
          const double vsignal = sound[i] + sound[j] - p.beta_visc * p.alpha_visc * dvdr;
          paux -= p.alpha_visc * vsignal * dvdr * winvrho;
          du -= 0.5 * m[j] * p.alpha_visc * vsignal * dvdr * dvdr * winvrho;
        }
        for (int k = 0; k < 3; k++) acc[k] += m[j] * dr[k] * paux;
      } else {
        // GradhSph::ComputeSphHydroGravForces
        double dr[3] = {draux[0], draux[1], draux[2]};
        double dv[3];
        for (int k = 0; k < 3; k++) dv[k] = v[k][j] - vi[k];
        const double drmag = std::sqrt(dot3(dr, dr) + kSmall);
        const double invdrmag = 1.0 / drmag;
        for (int k = 0; k < 3; k++) dr[k] *= invdrmag;
        const double dvdr = dot3(dv, dr);
        const double wi = hfactor[i] * w1(drmag * invh_i);
        const double wj = hfactor[j] * w1(drmag * invh_j);
        double paux = fac_i * wi + fac_j * wj;
        if (dvdr < 0.0) {
          const double winvrho = 0.25 * (wi + wj) * (invrho_i + invrho_j);
          const double vsignal = sound[i] + sound[j] - p.beta_visc * p.alpha_visc * dvdr;
          paux -= p.alpha_visc * vsignal * dvdr * winvrho;
          du -= 0.5 * m[j] * p.alpha_visc * vsignal * dvdr * dvdr * winvrho;
        }
        for (int k = 0; k < 3; k++) acc[k] += m[j] * dr[k] * paux;
        paux = 0.5 * (invhsqdi * wgrav(drmag * invh_i) + zeta[i] * wi +
                      invh_j * invh_j * wgrav(drmag * invh_j) + zeta[j] * wj);
        for (int k = 0; k < 3; k++) accg[k] += m[j] * dr[k] * paux;
        pot += 0.5 * m[j] * (invh_i * wpot(drmag * invh_i) + invh_j * wpot(drmag * invh_j));
        divv -= m[j] * dvdr * wi;
      }
    }
    divv *= invrho_i;
    du -= eos_pressure(rhoi, u[i]) * divv * invrho_i * invomega[i];
    if (!grav) {
      for (int k = 0; k < 3; k++) a[k][i] = acc[k];
      div_v[i] = divv; dudt[i] = du; gpot[i] = 0.0;
      for (int k = 0; k < 3; k++) ag[k][i] = 0.0;
    } else {
      for (int k = 0; k < 3; k++) { a[k][i] = acc[k]; ag[k][i] = accg[k]; }
      div_v[i] = divv; dudt[i] = du;
      gpot[i] += pot;
      // near candidates that are not SPH neighbours are direct-sum terms
      for (int q : direct_local) {
        const int j = cid[q];
        if (direct_out) direct_out->push_back(j);
        direct_term(i, cr[3 * q], cr[3 * q + 1], cr[3 * q + 2], m[j]);
      }
    }
  }

  // GradhSphBase::ComputeDirectGravForces, one term.
  void direct_term(int i, double rx, double ry, double rz, double mj) {
    double dr[3] = {rx - x[0][i], ry - x[1][i], rz - x[2][i]};
    const double drsqd = dot3(dr, dr) + kSmall;
    const double invdrmag = 1.0 / std::sqrt(drsqd);
    const double invdr3 = invdrmag * invdrmag * invdrmag;
    for (int k = 0; k < 3; k++) ag[k][i] += mj * dr[k] * invdr3;
    gpot[i] += mj * invdrmag;
  }

  // ---------------------------------------------------------------------------------
  // Hydro + self-gravity forces (open boundaries).
  void all_forces() {
    const bool quad = p.multipole == 1;
    begin_levels();
#pragma omp parallel
    {
      std::vector<int> near_id, direct_id, gcells;
      std::vector<double> near_r;
      int64_t local_pairs = 0, local_direct = 0, local_cells = 0;
      int* lv = thread_levels();
#pragma omp for schedule(guided)
      for (int li = 0; li < (int) leaves.size(); li++) {
        const int lc = leaves[li];
        const Cell& cell = cells[lc];
        if (!leaf_has_active(cell)) continue;
        near_id.clear(); near_r.clear(); direct_id.clear(); gcells.clear();
        const double hrangemax = kKernRange * cell.hmax, rmax = cell.rmax;
        const double hrangemaxsqd = std::pow(cell.rmax + kKernRange * cell.hmax, 2);
        walk([&](int cc, const Cell& o) -> int {
          double dr[3];
          for (int k = 0; k < 3; k++) dr[k] = o.rcell[k] - cell.rcell[k];
          const double drsqd = dot3(dr, dr);
          if (drsqd <= std::pow(o.rmax + rmax + hrangemax, 2) ||
              drsqd <= std::pow(rmax + o.rmax + kKernRange * o.hmax, 2)) {
            if (o.level < ltot) return 1;
            if (o.n == 0) return 0;
            for (int j = 0; j < o.n; j++) {
              const int id = order[o.first + j];
              double dd[3];
              for (int k = 0; k < 3; k++) dd[k] = x[k][id] - cell.rcell[k];
              const double ds = dot3(dd, dd);
              const double h2 = rmax + kKernRange * h[id];
              if (ds < hrangemaxsqd || ds < h2 * h2) {
                near_id.push_back(id);
                for (int k = 0; k < 3; k++) near_r.push_back(x[k][id]);
              } else {
                direct_id.push_back(id);   // demoted at the cell level (_EndSearch)
              }
            }
            return 0;
          }
          if (o.n == 0) return 0;
          if (!(drsqd < o.cdistsqd)) {           // geometric MAC: far enough
            if (o.level == ltot && o.n == 1) direct_id.push_back(order[o.first]);
            else gcells.push_back(cc);
            return 0;
          }
          if (o.level < ltot) return 1;
          for (int j = 0; j < o.n; j++) direct_id.push_back(order[o.first + j]);
          return 0;
        });
        if (want_lists) {
#pragma omp critical
          { gcell_leaf.push_back(lc); gcell_list.push_back(gcells); }
        }
        if (want_summary) {
          uint64_t hsh = 0;
          for (int cc : gcells) hsh += mix64((uint64_t) cc);
          cell_count[li] = (int64_t) gcells.size();
          cell_hash[li] = hsh;
        }
        int nact = 0;
        for (int j = 0; j < cell.n; j++) {
          const int i = order[cell.first + j];
          if (!is_active(i)) continue;
          nact++;
          gpot[i] = (m[i] / h[i]) * wpot(0.0);
          for (int k = 0; k < 3; k++) ag[k][i] = 0.0;
          std::vector<int> dl;
          const int64_t before = local_pairs;
          pair_loop(i, near_id, near_r, true, (want_lists || want_summary) ? &dl : nullptr, local_pairs, lv);
          local_direct += (int64_t) near_id.size() - (local_pairs - before);
          for (int id : direct_id) direct_term(i, x[0][id], x[1][id], x[2][id], m[id]);
          for (int cc : gcells) cell_term(i, cells[cc], quad);
          if (want_summary) {
            uint64_t hsh = 0;
            for (int id : dl) hsh += mix64((uint64_t) id);
            for (int id : direct_id) hsh += mix64((uint64_t) id);
            dir_count[i] = (int64_t) (dl.size() + direct_id.size());
            dir_hash[i] = hsh;
          }
          if (want_lists) {
            dl.insert(dl.end(), direct_id.begin(), direct_id.end());
            direct_neib[i] = dl;
          }
          for (int k = 0; k < 3; k++) a[k][i] += ag[k][i];
        }
        local_direct += (int64_t) nact * (int64_t) direct_id.size();
        local_cells += (int64_t) nact * (int64_t) gcells.size();
      }
#pragma omp atomic
      n_hydro_pairs += local_pairs;
#pragma omp atomic
      n_direct_pairs += local_direct;
#pragma omp atomic
      n_cell_pairs += local_cells;
    }
    end_levels();
  }

  // ComputeQuadropole<3> (NeighbourSearch.h:423-449) or the monopole sum (:349-377).
  void cell_term(int i, const Cell& c, bool quad) {
    double dr[3];
    if (quad) {
      for (int k = 0; k < 3; k++) dr[k] = x[k][i] - c.r[k];
      const double drsqd = dot3(dr, dr) + kSmall;
      const double invdrsqd = 1.0 / drsqd;
      const double invdrmag = std::sqrt(invdrsqd);
      const double invdr5 = invdrsqd * invdrsqd * invdrmag;
      for (int k = 0; k < 3; k++) ag[k][i] -= c.m * dr[k] * invdrsqd * invdrmag;
      const double* q = c.q;
      const double qscalar = q[0] * dr[0] * dr[0] + q[2] * dr[1] * dr[1] - (q[0] + q[2]) * dr[2] * dr[2] +
                             2.0 * (q[1] * dr[0] * dr[1] + q[3] * dr[0] * dr[2] + q[4] * dr[1] * dr[2]);
      const double qfactor = 2.5 * qscalar * invdr5 * invdrsqd;
      ag[0][i] += (q[0] * dr[0] + q[1] * dr[1] + q[3] * dr[2]) * invdr5 - qfactor * dr[0];
      ag[1][i] += (q[1] * dr[0] + q[2] * dr[1] + q[4] * dr[2]) * invdr5 - qfactor * dr[1];
      ag[2][i] += (q[3] * dr[0] + q[4] * dr[1] - (q[0] + q[2]) * dr[2]) * invdr5 - qfactor * dr[2];
      gpot[i] += c.m * invdrmag + 0.5 * qscalar * invdr5;
    } else {
      for (int k = 0; k < 3; k++) dr[k] = c.r[k] - x[k][i];
      const double drsqd = dot3(dr, dr) + kSmall;
      const double invdrsqd = 1.0 / drsqd;
      const double invdrmag = std::sqrt(invdrsqd);
      const double invdr3 = invdrsqd * invdrmag;
      gpot[i] += c.m * invdrmag;
      for (int k = 0; k < 3; k++) ag[k][i] += c.m * dr[k] * invdr3;
    }
  }

  // ---------------------------------------------------------------------------------
  // Gas <- stars: GradhSph::ComputeStarGravForces (src/GradhSph/GradhSph.cpp:698-743),
  // after gpot_hydro is taken (GradhSphTree.cpp:596-606; :385-391 in the hydro-only pass).
  void gas_from_stars() {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) {
      gpot_hydro[i] = gpot[i];
      if (nstar == 0) continue;
      double at[3] = {0.0, 0.0, 0.0}, pot = 0.0;
      for (int s_ = 0; s_ < nstar; s_++) {
        double dr[3];
        for (int k = 0; k < 3; k++) dr[k] = sx[k][s_] - x[k][i];
        const double drsqd = dot3(dr, dr) + kSmall;
        const double drmag = std::sqrt(drsqd);
        const double invdrmag = 1.0 / drmag;
        const double invhmean = 2.0 / (h[i] + sh[s_]);
        const double paux = sm[s_] * invhmean * invhmean * wgrav(drmag * invhmean) * invdrmag;
        for (int k = 0; k < 3; k++) at[k] += paux * dr[k];
        pot += sm[s_] * invhmean * wpot(drmag * invhmean);
      }
      for (int k = 0; k < 3; k++) { ag[k][i] += at[k]; a[k][i] += at[k]; }
      gpot[i] += pot;
    }
  }

  // Star <- gas: HydroTree::UpdateAllStarGasForces (src/Tree/HydroTree.cpp:551-654) with
  // Tree::ComputeStarGravityInteractionList (src/Tree/Tree.cpp:747-885) and
  // NbodyHermite4::CalculateDirectHydroForces (src/Nbody/NbodyHermite4.cpp:151-245).
  void stars_from_gas() {
    for (int k = 0; k < 3; k++) { s_a[k].assign(nstar, 0.0); s_adot[k].assign(nstar, 0.0); }
    s_gpot.assign(nstar, 0.0);
    const bool quad = p.multipole == 1;
#pragma omp parallel for schedule(dynamic)
    for (int s_ = 0; s_ < nstar; s_++) {
      const double rs[3] = {sx[0][s_], sx[1][s_], sx[2][s_]};
      const double vs[3] = {sv[0][s_], sv[1][s_], sv[2][s_]};
      const double hrangemax = kKernRange * sh[s_];
      std::vector<int> near_id, direct_id, gcells;
      walk([&](int cc, const Cell& o) -> int {
        double dr[3];
        for (int k = 0; k < 3; k++) dr[k] = o.rcell[k] - rs[k];
        const double drsqd = dot3(dr, dr);
        const double reach = 0.5 * hrangemax + o.rmax + 0.5 * kKernRange * o.hmax;
        if (drsqd < reach * reach) {
          if (o.level < ltot) return 1;
          for (int j = 0; j < o.n; j++) near_id.push_back(order[o.first + j]);
          return 0;
        }
        if (drsqd > o.cdistsqd && o.n > 0) {
          if (o.level == ltot && o.n == 1) direct_id.push_back(order[o.first]);
          else gcells.push_back(cc);
          return 0;
        }
        if (drsqd <= o.cdistsqd && o.n > 0) {
          if (o.level < ltot) return 1;
          for (int j = 0; j < o.n; j++) direct_id.push_back(order[o.first + j]);
        }
        return 0;
      });
      double acc[3] = {0.0, 0.0, 0.0}, adot[3] = {0.0, 0.0, 0.0}, pot = 0.0;
      for (int j : near_id) {
        double dr[3], dv[3];
        for (int k = 0; k < 3; k++) { dr[k] = x[k][j] - rs[k]; dv[k] = v[k][j] - vs[k]; }
        const double drsqd = dot3(dr, dr);
        const double drmag = std::sqrt(drsqd);
        const double invdrmag = 1.0 / drmag;
        const double invhmean = 2.0 / (sh[s_] + h[j]);
        const double drdt = dot3(dv, dr) * invdrmag;
        const double paux = m[j] * invhmean * invhmean * wgrav(drmag * invhmean) * invdrmag;
        const double wkern = w0(drmag * invhmean) * (double) std::pow((float) invhmean, 3.0f);
        for (int k = 0; k < 3; k++) acc[k] += paux * dr[k];
        for (int k = 0; k < 3; k++)
          adot[k] += paux * dv[k] - 3.0 * paux * drdt * invdrmag * dr[k] +
                     2.0 * kTwoPi * m[j] * drdt * wkern * invdrmag * dr[k];
        pot += m[j] * invhmean * wpot(drmag * invhmean);
      }
      for (int j : direct_id) {
        double dr[3], dv[3];
        for (int k = 0; k < 3; k++) { dr[k] = x[k][j] - rs[k]; dv[k] = v[k][j] - vs[k]; }
        const double drsqd = dot3(dr, dr);
        const double drmag = std::sqrt(drsqd);
        const double invdrmag = 1.0 / drmag;
        const double drdt = dot3(dv, dr) * invdrmag;
        const double inv3 = invdrmag * invdrmag * invdrmag;
        for (int k = 0; k < 3; k++) acc[k] += m[j] * dr[k] * inv3;
        for (int k = 0; k < 3; k++) adot[k] += m[j] * inv3 * (dv[k] - 3.0 * drdt * invdrmag * dr[k]);
        pot += m[j] * invdrmag;
      }
      for (int cc : gcells) {
        const Cell& c = cells[cc];
        double dr[3];
        if (quad) {
          for (int k = 0; k < 3; k++) dr[k] = rs[k] - c.r[k];
          const double drsqd = dot3(dr, dr) + kSmall;
          const double invdrsqd = 1.0 / drsqd;
          const double invdrmag = std::sqrt(invdrsqd);
          const double invdr5 = invdrsqd * invdrsqd * invdrmag;
          for (int k = 0; k < 3; k++) acc[k] -= c.m * dr[k] * invdrsqd * invdrmag;
          const double* q = c.q;
          const double qscalar = q[0] * dr[0] * dr[0] + q[2] * dr[1] * dr[1] - (q[0] + q[2]) * dr[2] * dr[2] +
                                 2.0 * (q[1] * dr[0] * dr[1] + q[3] * dr[0] * dr[2] + q[4] * dr[1] * dr[2]);
          const double qfactor = 2.5 * qscalar * invdr5 * invdrsqd;
          acc[0] += (q[0] * dr[0] + q[1] * dr[1] + q[3] * dr[2]) * invdr5 - qfactor * dr[0];
          acc[1] += (q[1] * dr[0] + q[2] * dr[1] + q[4] * dr[2]) * invdr5 - qfactor * dr[1];
          acc[2] += (q[3] * dr[0] + q[4] * dr[1] - (q[0] + q[2]) * dr[2]) * invdr5 - qfactor * dr[2];
          pot += c.m * invdrmag + 0.5 * qscalar * invdr5;
        } else {
          for (int k = 0; k < 3; k++) dr[k] = c.r[k] - rs[k];
          const double drsqd = dot3(dr, dr) + kSmall;
          const double invdrsqd = 1.0 / drsqd;
          const double invdrmag = std::sqrt(invdrsqd);
          pot += c.m * invdrmag;
          for (int k = 0; k < 3; k++) acc[k] += c.m * dr[k] * invdrsqd * invdrmag;
        }
      }
      for (int k = 0; k < 3; k++) { s_a[k][s_] = acc[k]; s_adot[k][s_] = adot[k]; }
      s_gpot[s_] = pot;
    }
  }

  // Set when the h solve's results are supplied by the caller (force pass only).
  bool given = false;
  std::vector<double> g_h, g_rho, g_invomega, g_zeta, g_pressure, g_sound;

  // ---------------------------------------------------------------------------------
  // KDK leapfrog with block timesteps: the gas part of SphSimulation::PostInitialConditionsSetup
  // and MainLoop (src/Hydrodynamics/SphSimulation.cpp:203-565, :573-880) with SphLeapfrogKDK
  // (src/Hydrodynamics/SphLeapfrogKDK.cpp:76-331), SphIntegration::Timestep
  // (src/Hydrodynamics/SphIntegration.cpp:81-130) and Simulation::ComputeBlockTimesteps
  // (src/Common/Simulation.cpp:1764-2190; ComputeGlobalTimestep :1664-1752 for one level).
  struct KdkParams { int32_t nlevels, level_diff_max, pad0, pad1; double courant_mult, accel_mult, energy_mult, pad2; };
  KdkParams kp{};
  bool energy_eq = false;
  int kn = 0, nresync = 0, level_max = 0, level_step = 1, Nsteps = 0;
  double t = 0.0, timestep = 0.0, dt_max = 0.0, timestep_old = 0.0;
  int64_t active_updates = 0;
  unsigned kdk_status = 0;       // 1 invalid timestep, 2 CheckTimesteps did not settle
  std::vector<double> r0[3], v0[3], a0[3], u0, dudt0, dt, dt_next, tlast;
  std::vector<int> nlast, nstep;
  std::vector<unsigned char> endstep;
  static int pow2i(int k) { return k >= 0 ? (1 << k) : 0; }   // (int) pow(2, k)

  // ComputeTimestepLevel, src/Headers/InlineFuncs.h:550-557
  static int timestep_level(double dt_, double dtmax) {
    const double kInvLogTwo = 1.44269504088896;   // invlogetwo, src/Headers/Constants.h:64
    const int l = (int) (kInvLogTwo * std::log(dtmax / dt_)) + 1;
    return l > 0 ? l : 0;
  }

  // SphIntegration::Timestep: Courant, acceleration and energy conditions
  double particle_timestep(int64_t i) {
    const double kSmallDp = 1.0e-50;   // small_number_dp, src/Headers/Constants.h:90
    const double hi = h[i];
    double ts = (kp.courant_mult * hi) / ((sound[i] + hi * std::fabs(div_v[i])) + kSmallDp);
    const double amag = std::sqrt((a[0][i] * a[0][i] + a[1][i] * a[1][i]) + a[2][i] * a[2][i]);
    ts = std::fmin(ts, kp.accel_mult * std::sqrt(hi / (amag + kSmallDp)));
    if (energy_eq) ts = std::fmin(ts, kp.energy_mult * (u[i] / (std::fabs(dudt[i]) + 1.0e-20)));
    if (!(ts <= 1.0e20) || !(ts > 0.0)) kdk_status |= 1u;
    return ts;
  }

  // GradhSph::ComputeThermalProperties for every particle before a force pass (the
  // radiation-step update of MainLoop, SphSimulation.cpp:672-679)
  void thermal_all() {
    const double gm1 = p.gamma_eos - 1.0;
    const double u_iso = p.temp0 / (p.gamma_eos - 1.0) / p.mu_bar;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) {
      if (p.eos == 1) u[i] = u_iso;
      sound[i] = p.eos == 1 ? std::sqrt(gm1 * u[i]) : std::sqrt(p.gamma_eos * gm1 * u[i]);
      pressure[i] = gm1 * rho[i] * u[i];
    }
  }

  // Tree build from the current positions and smoothing lengths.
  void kdk_build() {
    h_ghost = h;
    build_tree();
  }

  // One h solve (+ forces) over the active particles of the current tree.
  int kdk_pass(bool forces) {
    int64_t act = 0;
    for (int64_t i = 0; i < n; i++) act += active[i] ? 1 : 0;
    active_updates += act;
    const int st = density();
    if (st != 0) return st;
    update_hmax(0);
    thermal_all();
    if (forces) {
      if (p.self_gravity) all_forces(); else hydro_forces();
      // total acceleration written as the reference sums it (a + atree) by all_forces;
      // the hydro-only pass leaves atree zero
    }
    return 0;
  }

  void kdk_alloc() {
    for (int k = 0; k < 3; k++) { r0[k].assign(n, 0.0); v0[k].assign(n, 0.0); a0[k].assign(n, 0.0); }
    u0 = u; dudt0.assign(n, 0.0); dt.assign(n, 0.0); dt_next.assign(n, 0.0); tlast.assign(n, 0.0);
    nlast.assign(n, 0); nstep.assign(n, 0); level.assign(n, 0); levelneib.assign(n, 0);
    active.assign(n, 1); endstep.assign(n, 0);
    rho.assign(n, 0); invomega.assign(n, 1); zeta.assign(n, 0); hfactor.assign(n, 0);
    pressure.assign(n, 0); sound.assign(n, 0); div_v.assign(n, 0); dudt.assign(n, 0);
    gpot.assign(n, 0); hrangesqd.assign(n, 0); gpot_hydro.assign(n, 0);
    for (int k = 0; k < 3; k++) { a[k].assign(n, 0); ag[k].assign(n, 0); }
    kn = 0; nresync = 0; level_max = 0; level_step = 1; Nsteps = 0;
    t = timestep = dt_max = timestep_old = 0.0;
    active_updates = 0;
    kdk_status = 0;
  }

  // Simulation::ComputeBlockTimesteps (Nlevels > 1) / ComputeGlobalTimestep (Nlevels = 1)
  void block_timesteps() {
    const bool resync = kn == nresync;
    double dtmin = 9.9e99;
    int lmax_new = 0;
    // particles that start a new step (all of them when resynchronising)
    for (int64_t i = 0; i < n; i++) {
      if (kp.nlevels == 1 && !resync) continue;
      if (resync) {
        const double d = particle_timestep(i);
        dt_next[i] = d;
        dtmin = std::min(dtmin, d);
        continue;
      }
      const int dn = kn - nlast[i];
      if (dn == nstep[i] && nstep[i] != pow2i(level_step - level[i])) {
        // step shortened by CheckTimesteps (Saitoh & Makino)
        const double d = particle_timestep(i);
        const int lv = std::max(timestep_level(d, dt_max), levelneib[i] - kp.level_diff_max);
        level[i] = std::max(level[i], lv);
        levelneib[i] = level[i];
        nlast[i] = kn;
        nstep[i] = pow2i(level_step - level[i]);
        dt_next[i] = (double) nstep[i] * timestep;
        endstep[i] = 1;
      } else if (dn == nstep[i]) {
        const int ns = nstep[i], last_level = level[i];
        const double d = particle_timestep(i);
        const int lv = std::max(timestep_level(d, dt_max), levelneib[i] - kp.level_diff_max);
        int nl;
        if (lv < last_level && last_level > 1 && kn % (2 * ns) == 0) nl = last_level - 1;
        else if (lv > last_level) nl = lv;
        else nl = last_level;
        level[i] = nl;
        levelneib[i] = lv;
        nlast[i] = kn;
        nstep[i] = pow2i(level_step - nl);
        dt_next[i] = (double) nstep[i] * timestep;
        endstep[i] = 1;
      }
      lmax_new = std::max(lmax_new, level[i]);
    }
    // the integer-time state
    int up = 0, down = 0;
    if (kp.nlevels == 1) {
      if (resync) {
        kn = 0; level_max = 0; level_step = 0; nresync = 1;
        timestep = dtmin; timestep_old = timestep;
      }
    } else if (resync) {
      kn = 0;
      timestep = dtmin;
      level_max = kp.nlevels - 1;
      level_step = level_max;
      dt_max = dtmin * (double) pow2i(level_max);
      timestep_old = dtmin;
      nresync = pow2i(level_step);
      timestep = dt_max / (double) nresync;
    } else {
      const int level_max_old = level_max;
      const int istep = pow2i(level_step - level_max_old + 1);
      int lm;
      if (lmax_new > level_max_old) {
        const int nf = pow2i(lmax_new - level_max_old);
        kn *= nf; up = nf; lm = lmax_new;
      } else if (lmax_new <= level_max_old - 1 && level_max_old > 1 && istep > 0 && kn % istep == 0) {
        lm = level_max_old - 1;
        const int nf = pow2i(level_max_old - lm);
        kn /= nf; down = nf;
      } else {
        lm = level_max_old;
      }
      level_max = lm;
      level_step = lm;
      nresync = pow2i(level_step);
      timestep = dt_max / (double) nresync;
    }
    // levels after resynchronisation, or the rescaled integer steps
    for (int64_t i = 0; i < n; i++) {
      if (kp.nlevels == 1) {
        if (!resync) continue;
        endstep[i] = 1; level[i] = 0; levelneib[i] = 0; nstep[i] = 1; dt_next[i] = timestep_old;
        continue;
      }
      if (resync) {
        const int lv = std::min(timestep_level(dt_next[i], dt_max), level_max);
        level[i] = lv; levelneib[i] = lv;
        nstep[i] = pow2i(level_step - lv);
        nlast[i] = kn;
        dt_next[i] = (double) nstep[i] * timestep_old;
        endstep[i] = 1;
        continue;
      }
      if (up) { nstep[i] *= up; nlast[i] *= up; }
      if (down) { nlast[i] /= down; nstep[i] /= down; }
      if (nlast[i] == kn) nstep[i] = pow2i(level_step - level[i]);
    }
  }

  // SphLeapfrogKDK::EndTimestep (SphLeapfrogKDK.cpp:219-275)
  void end_timestep() {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) {
      if (!endstep[i]) continue;
      const double d = dt[i];
      for (int k = 0; k < 3; k++) {
        v[k][i] = v[k][i] + (0.5 * d) * (a[k][i] - a0[k][i]);
        r0[k][i] = x[k][i];
        v0[k][i] = v[k][i];
        a0[k][i] = a[k][i];
      }
      if (energy_eq) {
        double uu = u[i] + (0.5 * (dudt[i] - dudt0[i])) * d;
        if (uu <= 0.0) uu = u0[i] + dudt0[i] * d;
        u[i] = uu; u0[i] = uu; dudt0[i] = dudt[i];
      }
      nlast[i] = kn;
      tlast[i] = t;
      dt[i] = dt_next[i];
      dt_next[i] = 0.0;
      endstep[i] = 0;
      active[i] = 0;
    }
  }

  // Initial h solves, force pass and timesteps (PostInitialConditionsSetup with h provided).
  int kdk_setup() {
    kdk_alloc();
    kdk_build();
    int st = kdk_pass(false);
    if (st) return st;
    kdk_build();
    st = kdk_pass(true);
    if (st) return st;
    for (int64_t i = 0; i < n; i++) {
      for (int k = 0; k < 3; k++) { r0[k][i] = x[k][i]; v0[k][i] = v[k][i]; a0[k][i] = a[k][i]; }
      active[i] = 0;
    }
    block_timesteps();
    end_timestep();
    return 0;
  }

  // One MainLoop step.
  int kdk_step() {
    kn += 1; Nsteps += 1; t = t + timestep;
    // SphLeapfrogKDK::AdvanceParticles + TimeIntegration::CheckBoundaries
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) {
      const double d = t - tlast[i];
      for (int k = 0; k < 3; k++) {
        x[k][i] = (r0[k][i] + v0[k][i] * d) + ((0.5 * a0[k][i]) * d) * d;
        v[k][i] = v0[k][i] + a0[k][i] * d;
      }
      if (energy_eq) u[i] = u0[i] + dudt0[i] * d;
      active[i] = (kn - nlast[i] == nstep[i]) ? 1 : 0;
      if (p.periodic) {
        for (int k = 0; k < 3; k++) {
          const double L = p.boxmax[k] - p.boxmin[k];
          if (x[k][i] < p.boxmin[k]) { x[k][i] = x[k][i] + L; r0[k][i] = r0[k][i] + L; }
          if (x[k][i] > p.boxmax[k]) { x[k][i] = x[k][i] - L; r0[k][i] = r0[k][i] - L; }
        }
      }
    }
    kdk_build();
    const int kPasses = 3;   // the first pass and up to two CheckTimesteps repeats
    for (int pass = 0; pass < kPasses; pass++) {
      const int st = kdk_pass(true);
      if (st) return st;
      // unset active, then SphLeapfrogKDK::CheckTimesteps (SphLeapfrogKDK.cpp:284-331)
      int cnt = 0;
      for (int64_t i = 0; i < n; i++) {
        active[i] = 0;
        if (kp.nlevels <= 1) continue;
        const int dn = kn - nlast[i];
        if (dn != nstep[i] && levelneib[i] - level[i] > kp.level_diff_max) {
          const int level_new = levelneib[i] - kp.level_diff_max;
          const int nnewstep = pow2i(level_step - level_new);
          if (nnewstep > 0 && dn % nnewstep == 0) {
            if (dn > 0) nstep[i] = dn;
            level[i] = level_new;
            active[i] = 1;
            cnt++;
          }
        }
      }
      if (cnt == 0) break;
      if (pass == kPasses - 1) kdk_status |= 2u;
    }
    block_timesteps();
    end_timestep();
    return 0;
  }

  int run(int nthreads) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
    active.clear(); level.clear(); levelneib.clear();
    rho.assign(n, 0); invomega.assign(n, 1); zeta.assign(n, 0); hfactor.assign(n, 0);
    pressure.assign(n, 0); sound.assign(n, 0); div_v.assign(n, 0); dudt.assign(n, 0);
    gpot.assign(n, 0); hrangesqd.assign(n, 0); gpot_hydro.assign(n, 0);
    for (int k = 0; k < 3; k++) { a[k].assign(n, 0); ag[k].assign(n, 0); }
    if (want_lists || want_summary) hydro_neib.assign(n, {});
    if (want_lists) { direct_neib.assign(n, {}); gcell_list.clear(); gcell_leaf.clear(); }
    h_ghost = h;
    build_tree();
    if (want_summary) {
      dir_count.assign(n, 0); dir_hash.assign(n, 0);
      cell_count.assign(leaves.size(), 0); cell_hash.assign(leaves.size(), 0);
    }
    if (given) {
      // GradhSph::ComputeH's outputs taken as given (GradhSph.cpp:262-317)
      for (int64_t i = 0; i < n; i++) {
        h[i] = g_h[i]; rho[i] = g_rho[i]; invomega[i] = g_invomega[i]; zeta[i] = g_zeta[i];
        pressure[i] = g_pressure[i]; sound[i] = g_sound[i];
        const double invh = 1.0 / h[i];
        hfactor[i] = std::pow(invh, 3 + 1);
        hrangesqd[i] = kKernRangeSqd * h[i] * h[i];
        if (p.eos == 1) u[i] = p.temp0 / (p.gamma_eos - 1.0) / p.mu_bar;
      }
    } else {
      const int st = density();
      if (st != 0) return st;
    }
    update_hmax(0);
    if (p.self_gravity) all_forces(); else hydro_forces();
    gas_from_stars();
    if (nstar > 0 && p.self_gravity) stars_from_gas();
    return 0;
  }
};

}  // namespace

// ---- C entry points (ctypes) ------------------------------------------------------------
extern "C" {

enum { GSPH_ORACLE_NOUT = 20 };

int gsph_oracle_run(void* handle, int64_t n, const double* x, const double* y, const double* z,
                    const double* vx, const double* vy, const double* vz, const double* m,
                    const double* u, const double* h, int want_lists, int nthreads);

void* gsph_oracle_create(const Params* p) {
  Oracle* o = new Oracle();
  o->p = *p;
  return o;
}

void gsph_oracle_destroy(void* h) { delete static_cast<Oracle*>(h); }

// Run one step.  Arrays are in input order; returns 0 on success, -2 if an h iteration
// fails to converge (the reference raises an exception there).
int gsph_oracle_run(void* handle, int64_t n, const double* x, const double* y, const double* z,
                    const double* vx, const double* vy, const double* vz, const double* m,
                    const double* u, const double* h, int want_lists, int nthreads) {
  Oracle* o = static_cast<Oracle*>(handle);
  o->n = n;
  o->x[0].assign(x, x + n); o->x[1].assign(y, y + n); o->x[2].assign(z, z + n);
  o->v[0].assign(vx, vx + n); o->v[1].assign(vy, vy + n); o->v[2].assign(vz, vz + n);
  o->m.assign(m, m + n); o->u.assign(u, u + n); o->h.assign(h, h + n);
  o->want_lists = want_lists == 1;
  o->want_summary = want_lists == 2;
  o->n_density_pairs = o->n_hydro_pairs = o->n_direct_pairs = o->n_cell_pairs = 0;
  return o->run(nthreads);
}

// Force pass only: the h solve's results (h rho invomega zeta pressure sound, input
// order) are supplied instead of computed; the tree is built from the input h as usual.
int gsph_oracle_run_given(void* handle, int64_t n, const double* x, const double* y, const double* z,
                          const double* vx, const double* vy, const double* vz, const double* m,
                          const double* u, const double* h, const double* hs, const double* rho,
                          const double* invomega, const double* zeta, const double* pressure,
                          const double* sound, int want_lists, int nthreads) {
  Oracle* o = static_cast<Oracle*>(handle);
  o->given = true;
  o->g_h.assign(hs, hs + n); o->g_rho.assign(rho, rho + n); o->g_invomega.assign(invomega, invomega + n);
  o->g_zeta.assign(zeta, zeta + n); o->g_pressure.assign(pressure, pressure + n); o->g_sound.assign(sound, sound + n);
  const int st = gsph_oracle_run(handle, n, x, y, z, vx, vy, vz, m, u, h, want_lists, nthreads);
  o->given = false;
  return st;
}

// Per-particle results, n x 20 doubles in the order of oracle/refio.py PARTICLE_FIELDS.
void gsph_oracle_particles(void* handle, double* out) {
  Oracle* o = static_cast<Oracle*>(handle);
  for (int64_t i = 0; i < o->n; i++) {
    double* r = out + i * GSPH_ORACLE_NOUT;
    r[0] = o->h[i]; r[1] = o->rho[i]; r[2] = o->invomega[i]; r[3] = o->zeta[i];
    r[4] = o->hfactor[i]; r[5] = o->pressure[i]; r[6] = o->sound[i]; r[7] = o->u[i];
    r[8] = o->div_v[i]; r[9] = o->dudt[i];
    for (int k = 0; k < 3; k++) { r[10 + k] = o->a[k][i]; r[13 + k] = o->ag[k][i]; }
    r[16] = o->gpot[i]; r[17] = o->gpot_hydro[i]; r[18] = o->hrangesqd[i]; r[19] = 0.0;
  }
}

int gsph_oracle_ncell(void* handle) { return static_cast<Oracle*>(handle)->ncell; }
int gsph_oracle_ltot(void* handle) { return static_cast<Oracle*>(handle)->ltot; }

// Cell table in DFS order: N level m rmax hmax cdistsqd bbmin[3] bbmax[3] hbmin[3] hbmax[3]
// rcell[3] r[3] q[5]  (31 doubles per cell)
void gsph_oracle_cells(void* handle, double* out) {
  Oracle* o = static_cast<Oracle*>(handle);
  for (int c = 0; c < o->ncell; c++) {
    const Cell& cl = o->cells[c];
    double* r = out + (int64_t) c * 31;
    r[0] = cl.n; r[1] = cl.level; r[2] = cl.m; r[3] = cl.rmax; r[4] = cl.hmax; r[5] = cl.cdistsqd;
    for (int k = 0; k < 3; k++) {
      r[6 + k] = cl.bbmin[k]; r[9 + k] = cl.bbmax[k]; r[12 + k] = cl.hbmin[k]; r[15 + k] = cl.hbmax[k];
      r[18 + k] = cl.rcell[k]; r[21 + k] = cl.r[k];
    }
    for (int k = 0; k < 5; k++) r[24 + k] = cl.q[k];
    r[29] = cl.first; r[30] = 0;
  }
}

// Leaf-ordered particle ids (order[pos]).
void gsph_oracle_order(void* handle, int32_t* out) {
  Oracle* o = static_cast<Oracle*>(handle);
  for (int64_t i = 0; i < o->n; i++) out[i] = o->order[i];
}

// Lists: which = 0 hydro neighbours per particle, 1 direct-sum particles per particle,
// 2 gravity cells per active leaf (leaf ids via which = 3, one entry per leaf).
// Call with ids == nullptr to get the total size; off has (count + 1) entries.
int64_t gsph_oracle_list(void* handle, int which, int32_t* off, int32_t* ids) {
  Oracle* o = static_cast<Oracle*>(handle);
  const std::vector<std::vector<int>>* L = nullptr;
  if (which == 0) L = &o->hydro_neib;
  else if (which == 1) L = &o->direct_neib;
  else if (which == 2) L = &o->gcell_list;
  else if (which == 3) {
    if (ids) for (size_t i = 0; i < o->gcell_leaf.size(); i++) ids[i] = o->gcell_leaf[i];
    return (int64_t) o->gcell_leaf.size();
  }
  if (!L) return -1;
  int64_t tot = 0;
  for (const auto& v : *L) tot += (int64_t) v.size();
  if (!ids) return tot;
  int64_t pos = 0;
  off[0] = 0;
  for (size_t i = 0; i < L->size(); i++) {
    for (int id : (*L)[i]) ids[pos++] = id;
    off[i + 1] = (int32_t) pos;
  }
  return tot;
}

// Summaries of a run with want_lists == 2: direct partners per particle (input order)
// and multipole cells per leaf (left-to-right leaf order), as (count, hash).
void gsph_oracle_summary(void* handle, int64_t* dir_count, uint64_t* dir_hash, int32_t* leaf_cell,
                         int64_t* cell_count, uint64_t* cell_hash) {
  Oracle* o = static_cast<Oracle*>(handle);
  for (int64_t i = 0; i < o->n; i++) { dir_count[i] = o->dir_count[i]; dir_hash[i] = o->dir_hash[i]; }
  for (size_t q = 0; q < o->leaves.size(); q++) {
    leaf_cell[q] = o->leaves[q]; cell_count[q] = o->cell_count[q]; cell_hash[q] = o->cell_hash[q];
  }
}

// Star particles for the following runs (nstar = 0 removes them).
void gsph_oracle_set_stars(void* handle, int nstar, const double* x, const double* y, const double* z,
                           const double* vx, const double* vy, const double* vz, const double* m,
                           const double* h) {
  Oracle* o = static_cast<Oracle*>(handle);
  o->nstar = nstar;
  const double* r[3] = {x, y, z};
  const double* v[3] = {vx, vy, vz};
  for (int k = 0; k < 3; k++) { o->sx[k].assign(r[k], r[k] + nstar); o->sv[k].assign(v[k], v[k] + nstar); }
  o->sm.assign(m, m + nstar);
  o->sh.assign(h, h + nstar);
}

// Star results of the last run: nstar x 7 doubles (a[3], adot[3], gpot).
void gsph_oracle_stars(void* handle, double* out) {
  Oracle* o = static_cast<Oracle*>(handle);
  for (int s_ = 0; s_ < o->nstar; s_++) {
    double* r = out + (int64_t) s_ * 7;
    for (int k = 0; k < 3; k++) {
      r[k] = o->s_a[k].empty() ? 0.0 : o->s_a[k][s_];
      r[3 + k] = o->s_adot[k].empty() ? 0.0 : o->s_adot[k][s_];
    }
    r[6] = o->s_gpot.empty() ? 0.0 : o->s_gpot[s_];
  }
}

// One pass with block-timestep semantics, as a Simulation's main loop drives the neighbour
// search: a tree build (rebuild = 1) or the tree of the previous call (rebuild = 0, the
// repeated pass after CheckTimesteps, SphSimulation.cpp:641-752), the h solve of the active
// particles, the hmax update, the thermal update of every particle, and the force pass of
// the active particles.  Inactive particles keep the solved state given in `state`
// (n x 7: rho invomega zeta hfactor hrangesqd pressure sound); levelneib holds the values
// the records have before the force pass (active ones zeroed by Sph::ZeroAccelerations).
// Results as gsph_oracle_particles (levelneib in column 19).
int gsph_oracle_run_active(void* handle, int64_t n, const double* x, const double* y, const double* z,
                           const double* vx, const double* vy, const double* vz, const double* m,
                           const double* u, const double* h, const unsigned char* active, const int32_t* level,
                           const int32_t* levelneib, const double* state, int rebuild, int nthreads) {
  Oracle* o = static_cast<Oracle*>(handle);
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
  if (!rebuild && (o->n != n || o->cells.empty())) return -1;
  o->n = n;
  o->x[0].assign(x, x + n); o->x[1].assign(y, y + n); o->x[2].assign(z, z + n);
  o->v[0].assign(vx, vx + n); o->v[1].assign(vy, vy + n); o->v[2].assign(vz, vz + n);
  o->m.assign(m, m + n); o->u.assign(u, u + n); o->h.assign(h, h + n);
  o->want_lists = o->want_summary = false;
  o->active.assign(active, active + n);
  o->level.assign(level, level + n);
  o->levelneib.assign(levelneib, levelneib + n);
  std::vector<double>* st[7] = {&o->rho, &o->invomega, &o->zeta, &o->hfactor, &o->hrangesqd, &o->pressure, &o->sound};
  for (int q = 0; q < 7; q++) {
    st[q]->resize(n);
    for (int64_t i = 0; i < n; i++) (*st[q])[i] = state[i * 7 + q];
  }
  if (rebuild) {
    o->div_v.assign(n, 0); o->dudt.assign(n, 0); o->gpot.assign(n, 0); o->gpot_hydro.assign(n, 0);
    for (int k = 0; k < 3; k++) { o->a[k].assign(n, 0); o->ag[k].assign(n, 0); }
    o->h_ghost = o->h;
    o->build_tree();
  }
  o->n_density_pairs = o->n_hydro_pairs = o->n_direct_pairs = o->n_cell_pairs = 0;
  const int stt = o->density();
  if (stt != 0) return stt;
  o->update_hmax(0);
  o->thermal_all();
  if (o->p.self_gravity) o->all_forces(); else o->hydro_forces();
  o->gas_from_stars();
  return 0;
}

// Neighbour levels of the last run_active / KDK call (n ints).
void gsph_oracle_levelneib(void* handle, int32_t* out) {
  Oracle* o = static_cast<Oracle*>(handle);
  for (int64_t i = 0; i < o->n; i++) out[i] = o->levelneib.empty() ? 0 : o->levelneib[i];
}

// KDK run: SetupSimulation then nsteps main-loop steps of the gas with block timesteps.
// Inputs in input order.  out_state: n x 24 doubles (x y z vx vy vz ax ay az h rho u level
// nstep nlast levelneib dt tlast dudt div_v gpot invomega pressure sound); out_global: n t
// timestep level_max level_step nresync Nsteps dt_max; out_info: setup seconds, seconds of
// the nsteps steps, active updates of the setup, active updates of the steps, status.
// Returns 0, or -2 if an h iteration failed to converge.
int gsph_oracle_kdk(void* handle, int64_t n, const double* x, const double* y, const double* z,
                    const double* vx, const double* vy, const double* vz, const double* m,
                    const double* u, const double* h, const double* kdk_params, int nsteps, int nthreads,
                    double* out_state, double* out_global, double* out_info) {
  Oracle* o = static_cast<Oracle*>(handle);
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
  o->n = n;
  o->x[0].assign(x, x + n); o->x[1].assign(y, y + n); o->x[2].assign(z, z + n);
  o->v[0].assign(vx, vx + n); o->v[1].assign(vy, vy + n); o->v[2].assign(vz, vz + n);
  o->m.assign(m, m + n); o->u.assign(u, u + n); o->h.assign(h, h + n);
  o->want_lists = o->want_summary = false;
  o->kp = Oracle::KdkParams{};
  o->kp.nlevels = (int32_t) kdk_params[0];
  o->kp.level_diff_max = (int32_t) kdk_params[1];
  o->kp.courant_mult = kdk_params[2];
  o->kp.accel_mult = kdk_params[3];
  o->kp.energy_mult = kdk_params[4];
  o->energy_eq = o->p.eos == 0;
  o->n_density_pairs = o->n_hydro_pairs = o->n_direct_pairs = o->n_cell_pairs = 0;
  auto now = [] { return std::chrono::steady_clock::now(); };
  auto t0 = now();
  int st = o->kdk_setup();
  const double t_setup = std::chrono::duration<double>(now() - t0).count();
  const int64_t upd_setup = o->active_updates;
  auto t1 = now();
  for (int q = 0; q < nsteps && st == 0; q++) st = o->kdk_step();
  const double t_steps = std::chrono::duration<double>(now() - t1).count();
  if (out_info) {
    out_info[0] = t_setup; out_info[1] = t_steps;
    out_info[2] = (double) upd_setup; out_info[3] = (double) (o->active_updates - upd_setup);
    out_info[4] = (double) o->kdk_status;
  }
  if (st) return st;
  for (int64_t i = 0; i < n && out_state; i++) {
    double* r = out_state + i * 24;
    r[0] = o->x[0][i]; r[1] = o->x[1][i]; r[2] = o->x[2][i];
    r[3] = o->v[0][i]; r[4] = o->v[1][i]; r[5] = o->v[2][i];
    r[6] = o->a[0][i]; r[7] = o->a[1][i]; r[8] = o->a[2][i];
    r[9] = o->h[i]; r[10] = o->rho[i]; r[11] = o->u[i];
    r[12] = o->level[i]; r[13] = o->nstep[i]; r[14] = o->nlast[i]; r[15] = o->levelneib[i];
    r[16] = o->dt[i]; r[17] = o->tlast[i]; r[18] = o->dudt[i]; r[19] = o->div_v[i];
    r[20] = o->gpot[i]; r[21] = o->invomega[i]; r[22] = o->pressure[i]; r[23] = o->sound[i];
  }
  if (out_global) {
    out_global[0] = o->kn; out_global[1] = o->t; out_global[2] = o->timestep; out_global[3] = o->level_max;
    out_global[4] = o->level_step; out_global[5] = o->nresync; out_global[6] = o->Nsteps;
    out_global[7] = o->dt_max;
  }
  return 0;
}

int gsph_oracle_nleaf(void* handle) { return (int) static_cast<Oracle*>(handle)->leaves.size(); }

// Interaction counts of the last run: density pair evaluations, hydro pairs,
// direct pairs, cell-particle pairs.
void gsph_oracle_counts(void* handle, int64_t* out4) {
  Oracle* o = static_cast<Oracle*>(handle);
  out4[0] = o->n_density_pairs; out4[1] = o->n_hydro_pairs;
  out4[2] = o->n_direct_pairs; out4[3] = o->n_cell_pairs;
}

}  // extern "C"
