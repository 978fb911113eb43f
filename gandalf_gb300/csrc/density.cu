// Grad-h density and smoothing-length solve, one warp per leaf cell (fp64 form).
//
// Reference: GradhSphTree::UpdateAllSphProperties (src/GradhSph/GradhSphTree.cpp:82-271)
// drives, per active leaf cell, the gather walk Tree::ComputeGatherNeighbourList
// (src/Tree/Tree.cpp:290-381) and GradhSph::ComputeH (src/GradhSph/GradhSph.cpp:141-326).
//
// Mapping: lane = LPG * g + s.  Group g (LPG lanes) owns particle g of the leaf; the LPG
// lanes of a group split the candidate particles and reduce their sums with xor
// shuffles, so every lane of a group holds the same totals and runs the reference's
// scalar iteration logic in lock step.  The gather list (leaf cells overlapping the
// gather box, tagged with a periodic-image code) is staged in shared memory; a leaf
// whose list does not fit goes to the per-particle heavy-leaf kernel.  Each lane keeps
// (|r_ij|^2, m_j) of its candidates inside 2 hmax in its own compact list in global
// scratch, built once per attempt, and the iterations read it.  The warps are
// persistent and take leaves in depth-first order from a counter.
//
// The reference's retry protocol is kept: when any particle's h exceeds the cell's
// hmax (times 1.05 per attempt) the whole cell restarts from the input h with a 5 %
// larger hmax (GradhSphTree.cpp:154-240).
#include "gsph_state.cuh"
#include "gsph_walk.cuh"
#include "kernels.cuh"
#include "mixed_state.cuh"
#include "stars.cuh"

namespace gsph {

namespace {

constexpr int kDensStack = 1024;       // walk stack entries per warp
constexpr int kDensList = 1024;        // gather-list entries per warp
constexpr int kMaxAttempts = 256;      // attempts of the (skipping) hmax sequence
constexpr int kNodeBits = 25;          // depth-first ids < 2^25 (ltot <= 23)
constexpr int kNoShift = 13;           // periodic image code for (0,0,0)

__device__ __forceinline__ double shift_of(int code, int k, const SphParams& prm) {
  const int d = (k == 0 ? code % 3 : (k == 1 ? (code / 3) % 3 : code / 9)) - 1;
  return d == 0 ? 0.0 : (d > 0 ? prm.boxsize[k] : -prm.boxsize[k]);
}

template <int LPG>
__device__ __forceinline__ double group_sum(double v) {
#pragma unroll
  for (int o = 1; o < LPG; o <<= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}

// Final per-particle results of ComputeH (GradhSph.cpp:262-317).
__device__ __forceinline__ void write_density(const Particles& p, const SphParams& prm, int slot, double hfin,
                                              double rho_out, double om_out, double zeta_out, double xi, double yi,
                                              double zi) {
  const double invh = 1.0 / hfin;
  p.h[slot] = hfin;
  p.rho[slot] = rho_out;
  p.hfactor[slot] = invh * invh * invh * invh;
  p.hrangesqd[slot] = __dmul_rn(__dmul_rn(kKernRangeSqd, hfin), hfin);
  p.div_v[slot] = 0.0;
  const double drho = -(1.0 / 3.0) * hfin / rho_out;   // h_rho_deriv, src/Headers/Sph.h:264-268
  const double io = 1.0 / (1.0 - drho * om_out);
  p.invomega[slot] = io;
  const double zsum = prm.stars.n ? zeta_out + star_zeta_sum(prm.stars, xi, yi, zi, hfin) : zeta_out;
  p.zeta[slot] = drho * zsum * io;
  double u = p.u[slot];
  const double gm1 = prm.gamma_eos - 1.0;
  if (prm.eos == 1) { u = prm.u_iso; p.u[slot] = u; }
  p.sound[slot] = prm.eos == 1 ? sqrt(gm1 * u) : sqrt(prm.gamma_eos * gm1 * u);
  p.pressure[slot] = gm1 * rho_out * u;
}

// Per-lane compact lists of (|dr|^2, m) for the candidates inside 2 hmax_list, built once
// per attempt in global scratch (one region per resident warp): every iteration then reads
// the lane's own list instead of recomputing |dr|^2 of every candidate.  Each lane keeps
// its candidates in the order it visits them, so the sums are the same, bit for bit, as
// the rescanning form; a lane whose list overflows rescans.
constexpr int kCompLane = 64;                              // entries per lane
constexpr int kCompWarp = 32 * kCompLane;                  // double2 entries per warp
constexpr int kDensResident = 152 * 16;                    // persistent warps (blocks)

template <int LPG>
__device__ __forceinline__ void density_leaf_fp64(const Tree& t, const Particles& p, const SphParams& prm,
                                                  const DeviceCounters& cnt, const HeavyList& heavy, int leaf,
                                                  int* stack, int* list, double2* comp) {
  const int lane = threadIdx.x & 31;
  const int g = lane / LPG, sl = lane % LPG;
  const int c = t.leaf_cell[leaf];
  const int first = t.cell_first[c], ncell = t.cell_n[c];
  const bool mine = g < ncell && is_active(p, first + g);
  if (!__any_sync(kFull, mine)) return;   // no active particle in this leaf
  const int slot = first + (g < ncell ? g : 0);
  const double xi = p.x[slot], yi = p.y[slot], zi = p.z[slot], mi = p.m[slot];
  const double h_start = p.h[slot];
  const CellBox bb = t.bb[c];
  double hmax = t.geom[c].hmax;
  unsigned long long pairs = 0;

  // final per-particle results
  double h_out = h_start, rho_out = 0.0, om_out = 0.0, zeta_out = 0.0, hl_out = 0.0;
  bool fail = false, stack_ok = true;

  // One attempt of the reference's cell loop with gather radius 2*hmax_list.
  // GradhSph::ComputeH with hmax = hmax_list for every particle of the cell; returns
  // true if some particle's h exceeded hmax (the cell must be redone).  mcheck keeps
  // the largest h the reference's "h > hmax" test has seen.  (probe == true stops
  // after the fixed-point phase.)
  double mcheck = 0.0;
  bool gave_up = false;   // gather list too long for one warp: the leaf goes to the heavy kernel
  auto attempt = [&](double hmax_list, bool probe) -> bool {
    const double hr = __dmul_rn(kKernRange, hmax_list);
    double gmin[3], gmax[3];
    for (int k = 0; k < 3; k++) { gmin[k] = __dsub_rn(bb.bbmin[k], hr); gmax[k] = __dadd_rn(bb.bbmax[k], hr); }
    int nsh[3] = {1, 1, 1}, sh[3][3];
    for (int k = 0; k < 3; k++) {
      sh[k][0] = 1;
      if (prm.periodic) {
        if (gmax[k] > prm.boxmax[k]) sh[k][nsh[k]++] = 2;   // images r + L of lhs particles
        if (gmin[k] < prm.boxmin[k]) sh[k][nsh[k]++] = 0;   // images r - L of rhs particles
      }
    }
    WarpLists L{list, list, list, 0, 0, 0, kDensList};
    bool overflow = false;
    auto walk_all = [&](auto&& flush) {
      for (int a0 = 0; a0 < nsh[0]; a0++)
        for (int a1 = 0; a1 < nsh[1]; a1++)
          for (int a2 = 0; a2 < nsh[2]; a2++) {
            const int code = sh[0][a0] + 3 * sh[1][a1] + 9 * sh[2][a2];
            double bmin[3], bmax[3];
            for (int k = 0; k < 3; k++) {
              const double s = shift_of(code, k, prm);
              bmin[k] = gmin[k] - s;
              bmax[k] = gmax[k] - s;
            }
            auto decide = [&](int node, int level) -> int {
              const CellBox ob = t.bb[node];
              if (t.cell_n[node] == 0) return kSkip;
              if (!box_overlap(bmin, bmax, ob.bbmin, ob.bbmax)) return kSkip;
              return level == t.ltot ? kEmitA : kOpen;
            };
            auto tag = [&](int node, int) { return node | (code << kNodeBits); };
            stack_ok = stack_ok && warp_walk(0, t.ltot, t.cell_level, stack, kDensStack, L, decide, tag, flush);
          }
    };
    walk_all([&]() { overflow = true; });
    if (overflow && heavy.leaves) { gave_up = true; return false; }
    const int ncached = L.na;

    // |dr|^2 exactly as the iteration computes it; every pair inside the kernel support
    // of an h <= hmax_list has |dr|^2 < 4 hmax_list^2 (the margin covers the roundings)
    int ncomp = 0;
    if (!overflow && mine) {
      const double lim = 4.0 * hmax_list * hmax_list * (1.0 + 1.0e-12);
      for (int e = 0; e < ncached; e++) {
        const int tagv = list[e];
        const int node = tagv & ((1 << kNodeBits) - 1);
        const int code = tagv >> kNodeBits;
        const int f = t.cell_first[node], nn = t.cell_n[node];
        const double sx = shift_of(code, 0, prm), sy = shift_of(code, 1, prm), sz = shift_of(code, 2, prm);
        for (int q = sl; q < nn; q += LPG) {
          const int j = f + q;
          double xj = p.x[j], yj = p.y[j], zj = p.z[j];
          if (code != kNoShift) {
            const double glim = __dmul_rn(kGhostRange * kKernRange, p.h0[j]);
            bool ok = true;
            if (sx > 0.0) ok = ok && (xj < __dadd_rn(prm.boxmin[0], glim));
            if (sx < 0.0) ok = ok && (xj > __dsub_rn(prm.boxmax[0], glim));
            if (sy > 0.0) ok = ok && (yj < __dadd_rn(prm.boxmin[1], glim));
            if (sy < 0.0) ok = ok && (yj > __dsub_rn(prm.boxmax[1], glim));
            if (sz > 0.0) ok = ok && (zj < __dadd_rn(prm.boxmin[2], glim));
            if (sz < 0.0) ok = ok && (zj > __dsub_rn(prm.boxmax[2], glim));
            if (!ok) continue;
            xj = __dadd_rn(xj, sx); yj = __dadd_rn(yj, sy); zj = __dadd_rn(zj, sz);
          }
          const double dx = xj - xi, dy = yj - yi, dz = zj - zi;
          const double drsqd = dot3_rn(dx, dy, dz);
          if (drsqd <= lim) {
            if (ncomp < kCompLane) comp[(g * kCompLane + ncomp) * LPG + sl] = make_double2(drsqd, p.m[j]);
            ncomp++;
          }
        }
      }
    }
    const bool use_comp = !overflow && ncomp <= kCompLane;

    double hi = h_start, h_lower = 0.0, h_upper = hmax_list;
    double rho = 0.0, om = 0.0, zeta = 0.0;
    int iteration = 0;
    bool done = !mine, abort_cell = false;
    double mloc = 0.0;
    while (__any_sync(kFull, !done)) {
      iteration++;
      const double invh = 1.0 / hi;
      const double invhsqd = invh * invh;
      double srho = 0.0, som = 0.0, sze = 0.0;
      auto consume = [&](int count) {
        if (done) return;
        for (int e = 0; e < count; e++) {
          const int tagv = list[e];
          const int node = tagv & ((1 << kNodeBits) - 1);
          const int code = tagv >> kNodeBits;
          const int f = t.cell_first[node], nn = t.cell_n[node];
          const double sx = shift_of(code, 0, prm), sy = shift_of(code, 1, prm), sz = shift_of(code, 2, prm);
          for (int q = sl; q < nn; q += LPG) {
            const int j = f + q;
            double xj = p.x[j], yj = p.y[j], zj = p.z[j];
            if (code != kNoShift) {
              const double lim = __dmul_rn(kGhostRange * kKernRange, p.h0[j]);
              bool ok = true;
              if (sx > 0.0) ok = ok && (xj < __dadd_rn(prm.boxmin[0], lim));
              if (sx < 0.0) ok = ok && (xj > __dsub_rn(prm.boxmax[0], lim));
              if (sy > 0.0) ok = ok && (yj < __dadd_rn(prm.boxmin[1], lim));
              if (sy < 0.0) ok = ok && (yj > __dsub_rn(prm.boxmax[1], lim));
              if (sz > 0.0) ok = ok && (zj < __dadd_rn(prm.boxmin[2], lim));
              if (sz < 0.0) ok = ok && (zj > __dsub_rn(prm.boxmax[2], lim));
              if (!ok) continue;
              xj = __dadd_rn(xj, sx); yj = __dadd_rn(yj, sy); zj = __dadd_rn(zj, sz);
            }
            const double dx = xj - xi, dy = yj - yi, dz = zj - zi;
            const double ssqd = invhsqd * dot3_rn(dx, dy, dz);
            if (ssqd < kKernRangeSqd) {
              const double s = sqrt(ssqd);
              const double mj = p.m[j];
              srho = fma(mj, m4_w0(s), srho);
              som = fma(mj * invh, m4_womega(s), som);
              sze = fma(mj, m4_wzeta(s), sze);
              pairs++;
            }
          }
        }
      };
      if (use_comp) {
        if (!done) {
          for (int k = 0; k < ncomp; k++) {
            const double2 v = comp[(g * kCompLane + k) * LPG + sl];
            const double ssqd = invhsqd * v.x;
            if (ssqd < kKernRangeSqd) {
              const double s = sqrt(ssqd);
              srho = fma(v.y, m4_w0(s), srho);
              som = fma(v.y * invh, m4_womega(s), som);
              sze = fma(v.y, m4_wzeta(s), sze);
              pairs++;
            }
          }
        }
      } else if (!overflow) {
        consume(ncached);
      } else {
        L = WarpLists{list, list, list, 0, 0, 0, kDensList};
        walk_all([&]() { consume(L.na); });
        consume(L.na);
      }
      srho = group_sum<LPG>(srho);
      som = group_sum<LPG>(som);
      sze = group_sum<LPG>(sze);
      if (!done) {
        const double hfac3 = invh * invh * invh;
        rho = srho * hfac3;
        om = som * hfac3;
        zeta = sze * invhsqd;
        const double hrho = prm.h_fac * pow(mi / rho, 1.0 / 3.0);
        if (rho > 0.0 && hi > h_lower && fabs(hi - hrho) * invh < prm.h_converge) {
          done = true;
        } else if (probe && iteration >= 30) {
          done = true;                      // the bisection phase never exceeds hmax
        } else {
          if (iteration < 30) hi = hrho;
          else if (iteration == 30) hi = 0.5 * (h_lower + h_upper);
          else if (iteration < 150) {
            if (rho < kSmall || hi > hrho) h_upper = hi; else h_lower = hi;
            hi = 0.5 * (h_lower + h_upper);
          } else {
            fail = true;
            done = true;
          }
          if (!done) {
            mloc = fmax(mloc, hi);
            if (hi > hmax_list) { abort_cell = true; done = true; }
            else if (!(hi > h_lower && hi < h_upper)) done = true;
          }
        }
      }
    }
    double mw = mloc;
    for (int o = 16; o > 0; o >>= 1) mw = fmax(mw, __shfl_xor_sync(kFull, mw, o));
    mcheck = fmax(mcheck, mw);
    const bool any_abort = __any_sync(kFull, abort_cell);
    if (!any_abort && !probe && mine) {
      h_out = fmax(prm.h_fac * pow(mi / rho, 1.0 / 3.0), h_lower);
      rho_out = rho; om_out = om; zeta_out = zeta; hl_out = h_lower;
    }
    return any_abort;
  };

  // Reference sequence: hmax_k = 1.05 hmax_{k-1}, redo the cell while some h > hmax_k
  // (GradhSphTree.cpp:154-240).  The h values an attempt visits before its abort do not
  // depend on hmax_k, so every hmax_j below the largest h seen so far would abort too:
  // the next attempt jumps to the first hmax_j of the same sequence at or above it.
  bool solved = false;
  double hk = __dmul_rn(1.05, hmax);
  for (int a = 0; a < kMaxAttempts && !solved; a++) {
    if (!attempt(hk, false)) {
      if (gave_up) break;
      solved = true;
    } else {
      int guard = 0;
      do { hk = __dmul_rn(1.05, hk); } while (hk < mcheck && ++guard < 100000);
    }
  }
  if (gave_up) {   // nothing written; the heavy kernel solves the leaf from the start
    if (lane == 0) {
      const int k = atomicAdd(heavy.count, 1);
      heavy.leaves[k] = leaf;
    }
    return;
  }
  if (!stack_ok && lane == 0) atomicOr(cnt.status, (unsigned) kStatusStackOverflow);
  if (__any_sync(kFull, fail) && lane == 0) atomicOr(cnt.status, (unsigned) kStatusHNotConverged);
  if (!solved && lane == 0) atomicOr(cnt.status, (unsigned) kStatusRetryLimit);
  {
    unsigned long long tot = pairs;
    for (int o = 16; o > 0; o >>= 1) tot += __shfl_xor_sync(kFull, tot, o);
    if (lane == 0) atomicAdd(cnt.density_pairs, tot);
  }
  if (mine && sl == 0) write_density(p, prm, slot, h_out, rho_out, om_out, zeta_out, xi, yi, zi);
}

// Persistent warps (one per block) take leaves in depth-first order from a counter.
template <int LPG>
__global__ void __launch_bounds__(32, 16)
k_density_fp64(Tree t, Particles p, SphParams prm, DeviceCounters cnt, HeavyList heavy, int* next,
               double2* scratch) {
  __shared__ int s_stack[kDensStack];
  __shared__ int s_list[kDensList];
  double2* comp = scratch + (size_t) blockIdx.x * kCompWarp;
  const int lane = threadIdx.x & 31;
  for (;;) {
    int leaf = 0;
    if (lane == 0) leaf = atomicAdd(next, 1);
    leaf = __shfl_sync(kFull, leaf, 0);
    if (leaf >= t.nleaf) break;
    density_leaf_fp64<LPG>(t, p, prm, cnt, heavy, leaf, s_stack, s_list, comp);
    __syncwarp();
  }
}


// ---- heavy leaves ----------------------------------------------------------------------
// One block per leaf, one warp per particle; each h iteration walks the tree for the
// particle's own box r +- 2h (a superset: the exact FP64 test below decides every pair),
// instead of scanning the leaf's whole gather list.  Every pair inside the kernel support
// of the current h lies inside the leaf's gather box while h stays below hmax_list, so the
// sums take the same pairs as the warp-per-leaf form; the cell-level attempt protocol is
// kept across the block.
constexpr int kPPStack = 1024;
constexpr int kPPList = 256;

struct PPShared64 {
  int stack[8][kPPStack];
  int list[8][kPPList];
  double h0[32];
  double mloc[8];
};

template <int LPG>
__device__ __forceinline__ void density_pp_leaf_fp64(const Tree& t, const Particles& p, const SphParams& prm,
                                                     const DeviceCounters& cnt, int leaf, PPShared64& sm) {
  constexpr int G = 32 / LPG;
  const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int* stack = sm.stack[wib];
  int* list = sm.list[wib];
  unsigned long long pairs = 0;
  bool stack_ok = true, fail = false;
  const int c = t.leaf_cell[leaf];
  const int first = t.cell_first[c], ncell = t.cell_n[c];
  __syncthreads();
  if (threadIdx.x < ncell) sm.h0[threadIdx.x] = p.h[first + threadIdx.x];
  __syncthreads();
  double hk = __dmul_rn(1.05, t.geom[c].hmax);
  bool solved = false;
  for (int att = 0; att < kMaxAttempts && !solved; att++) {
    double mloc = 0.0;
    bool abort_any = false;
    for (int g = wib; g < ncell; g += 8) {
      const int slot = first + g;
      if (!is_active(p, slot)) continue;
      const double xi = p.x[slot], yi = p.y[slot], zi = p.z[slot], mi = p.m[slot];
      double hi = sm.h0[g], h_lower = 0.0, h_upper = hk;
      double rho = 0.0, om = 0.0, zeta = 0.0;
      bool done = false, abort_cell = false;
      int iteration = 0;
      while (!done) {
        iteration++;
        const double invh = 1.0 / hi;
        const double invhsqd = invh * invh;
        double srho = 0.0, som = 0.0, sze = 0.0;
        const double rr = __dmul_rn(kKernRange * (1.0 + 1.0 / 1024.0), hi);
        const double gmin[3] = {xi - rr, yi - rr, zi - rr}, gmax[3] = {xi + rr, yi + rr, zi + rr};
        int nsh[3] = {1, 1, 1}, sh[3][3];
        for (int q = 0; q < 3; q++) {
          sh[q][0] = 1;
          if (prm.periodic) {
            if (gmax[q] > prm.boxmax[q]) sh[q][nsh[q]++] = 2;
            if (gmin[q] < prm.boxmin[q]) sh[q][nsh[q]++] = 0;
          }
        }
        WarpLists L{list, list, list, 0, 0, 0, kPPList};
        auto consume = [&]() {
          for (int e0 = 0; e0 < L.na; e0 += LPG) {
            const int e = e0 + lane / G, q = lane % G;
            if (e >= L.na) continue;
            const int tagv = list[e];
            const int node = tagv & ((1 << kNodeBits) - 1);
            const int code = tagv >> kNodeBits;
            if (q >= t.cell_n[node]) continue;
            const int j = t.cell_first[node] + q;
            double xj = p.x[j], yj = p.y[j], zj = p.z[j];
            if (code != kNoShift) {
              const double sx = shift_of(code, 0, prm), sy = shift_of(code, 1, prm), sz = shift_of(code, 2, prm);
              const double lim = __dmul_rn(kGhostRange * kKernRange, p.h0[j]);
              bool ok = true;
              if (sx > 0.0) ok = ok && (xj < __dadd_rn(prm.boxmin[0], lim));
              if (sx < 0.0) ok = ok && (xj > __dsub_rn(prm.boxmax[0], lim));
              if (sy > 0.0) ok = ok && (yj < __dadd_rn(prm.boxmin[1], lim));
              if (sy < 0.0) ok = ok && (yj > __dsub_rn(prm.boxmax[1], lim));
              if (sz > 0.0) ok = ok && (zj < __dadd_rn(prm.boxmin[2], lim));
              if (sz < 0.0) ok = ok && (zj > __dsub_rn(prm.boxmax[2], lim));
              if (!ok) continue;
              xj = __dadd_rn(xj, sx); yj = __dadd_rn(yj, sy); zj = __dadd_rn(zj, sz);
            }
            const double dx = xj - xi, dy = yj - yi, dz = zj - zi;
            const double ssqd = invhsqd * dot3_rn(dx, dy, dz);
            if (ssqd < kKernRangeSqd) {
              const double sv = sqrt(ssqd);
              const double mj = p.m[j];
              srho = fma(mj, m4_w0(sv), srho);
              som = fma(mj * invh, m4_womega(sv), som);
              sze = fma(mj, m4_wzeta(sv), sze);
              pairs++;
            }
          }
          __syncwarp();
        };
        for (int a0 = 0; a0 < nsh[0]; a0++)
          for (int a1 = 0; a1 < nsh[1]; a1++)
            for (int a2 = 0; a2 < nsh[2]; a2++) {
              const int code = sh[0][a0] + 3 * sh[1][a1] + 9 * sh[2][a2];
              double bmin[3], bmax[3];
              for (int q = 0; q < 3; q++) {
                const double sft = shift_of(code, q, prm);
                bmin[q] = gmin[q] - sft;
                bmax[q] = gmax[q] - sft;
              }
              auto decide = [&](int node, int level) -> int {
                if (t.cell_n[node] == 0) return kSkip;
                const CellBox ob = t.bb[node];
                if (!box_overlap(bmin, bmax, ob.bbmin, ob.bbmax)) return kSkip;
                return level == t.ltot ? kEmitA : kOpen;
              };
              auto tag = [&](int node, int) { return node | (code << kNodeBits); };
              stack_ok = warp_walk(0, t.ltot, t.cell_level, stack, kPPStack, L, decide, tag, consume) && stack_ok;
              consume();
              L.na = 0;
            }
        for (int o = 16; o > 0; o >>= 1) {
          srho += __shfl_xor_sync(kFull, srho, o);
          som += __shfl_xor_sync(kFull, som, o);
          sze += __shfl_xor_sync(kFull, sze, o);
        }
        // GradhSph::ComputeH iteration (as the warp-per-leaf kernel)
        const double hfac3 = invh * invh * invh;
        rho = srho * hfac3;
        om = som * hfac3;
        zeta = sze * invhsqd;
        const double hrho = prm.h_fac * pow(mi / rho, 1.0 / 3.0);
        if (rho > 0.0 && hi > h_lower && fabs(hi - hrho) * invh < prm.h_converge) {
          done = true;
        } else {
          if (iteration < 30) hi = hrho;
          else if (iteration == 30) hi = 0.5 * (h_lower + h_upper);
          else if (iteration < 150) {
            if (rho < kSmall || hi > hrho) h_upper = hi; else h_lower = hi;
            hi = 0.5 * (h_lower + h_upper);
          } else {
            fail = true;
            done = true;
          }
          if (!done) {
            mloc = fmax(mloc, hi);
            if (hi > hk) { abort_cell = true; done = true; }
            else if (!(hi > h_lower && hi < h_upper)) done = true;
          }
        }
        if (!stack_ok) done = true;
      }
      abort_any = abort_any || abort_cell;
      if (!abort_cell && lane == 0) {
        const double hfin = fmax(prm.h_fac * pow(mi / rho, 1.0 / 3.0), h_lower);
        write_density(p, prm, slot, hfin, rho, om, zeta, xi, yi, zi);
      }
    }
    if (lane == 0) sm.mloc[wib] = mloc;
    abort_any = __syncthreads_or(abort_any);
    if (!abort_any) { solved = true; break; }
    double mc = 0.0;
    for (int w = 0; w < 8; w++) mc = fmax(mc, sm.mloc[w]);
    __syncthreads();
    int guard = 0;
    do { hk = __dmul_rn(1.05, hk); } while (hk < mc && ++guard < 100000);
  }
  unsigned long long tot = pairs;
  for (int o = 16; o > 0; o >>= 1) tot += __shfl_xor_sync(kFull, tot, o);
  if (lane == 0) {
    if (tot) atomicAdd(cnt.density_pairs, tot);
    if (!stack_ok) atomicOr(cnt.status, (unsigned) kStatusStackOverflow);
    if (fail) atomicOr(cnt.status, (unsigned) kStatusHNotConverged);
    if (!solved && wib == 0) atomicOr(cnt.status, (unsigned) kStatusRetryLimit);
  }
}

template <int LPG>
__global__ void __launch_bounds__(256, 2) k_density_fp64_pp(Tree t, Particles p, SphParams prm, DeviceCounters cnt,
                                                            HeavyList heavy) {
  __shared__ PPShared64 sm;
  const int nh = *heavy.count;
  for (int k = blockIdx.x; k < nh; k += gridDim.x) density_pp_leaf_fp64<LPG>(t, p, prm, cnt, heavy.leaves[k], sm);
}

}  // namespace

size_t density_fp64_scratch_entries() { return (size_t) kDensResident * kCompWarp; }

void launch_density(const Tree& t, const Particles& p, const SphParams& prm, const DeviceCounters& cnt,
                    const HeavyList& heavy, int lanes_per_particle, int* next, double2* scratch, cudaStream_t st) {
  cudaMemsetAsync(heavy.count, 0, sizeof(int), st);
  cudaMemsetAsync(next, 0, sizeof(int), st);
  const int blocks = kDensResident < t.nleaf ? kDensResident : t.nleaf;
  switch (lanes_per_particle) {
    case 32: k_density_fp64<32><<<blocks, 32, 0, st>>>(t, p, prm, cnt, heavy, next, scratch); break;
    case 16: k_density_fp64<16><<<blocks, 32, 0, st>>>(t, p, prm, cnt, heavy, next, scratch); break;
    case 8: k_density_fp64<8><<<blocks, 32, 0, st>>>(t, p, prm, cnt, heavy, next, scratch); break;
    case 4: k_density_fp64<4><<<blocks, 32, 0, st>>>(t, p, prm, cnt, heavy, next, scratch); break;
    case 2: k_density_fp64<2><<<blocks, 32, 0, st>>>(t, p, prm, cnt, heavy, next, scratch); break;
    default: k_density_fp64<1><<<blocks, 32, 0, st>>>(t, p, prm, cnt, heavy, next, scratch); break;
  }
  const int gpp = 2 * 152;
  switch (lanes_per_particle) {
    case 32: k_density_fp64_pp<32><<<gpp, 256, 0, st>>>(t, p, prm, cnt, heavy); break;
    case 16: k_density_fp64_pp<16><<<gpp, 256, 0, st>>>(t, p, prm, cnt, heavy); break;
    case 8: k_density_fp64_pp<8><<<gpp, 256, 0, st>>>(t, p, prm, cnt, heavy); break;
    case 4: k_density_fp64_pp<4><<<gpp, 256, 0, st>>>(t, p, prm, cnt, heavy); break;
    case 2: k_density_fp64_pp<2><<<gpp, 256, 0, st>>>(t, p, prm, cnt, heavy); break;
    default: k_density_fp64_pp<1><<<gpp, 256, 0, st>>>(t, p, prm, cnt, heavy); break;
  }
}

}  // namespace gsph
