// Mixed-precision form of the per-leaf kernels: fp32 pair arithmetic and kernel sums, an
// fp64 h-rho iteration state and convergence test, fp64 positions and cell moments (kept
// as float hi/lo pairs for the pair loops), and interaction lists identical to the fp64 form.
//
// Pair formulas are those of the fp64 kernels (density.cu, forces.cu; reference
// src/GradhSph/GradhSph.cpp:141-690, src/Headers/NeighbourSearch.h:423-449) evaluated in
// float.  Every membership decision — tree-walk near test and multipole acceptance
// (src/Tree/Tree.cpp:627-735), SPH-neighbour test (src/Headers/NeighbourManager.h:521) —
// is made in float with relative margin kMargin and re-made with the reference's fp64
// arithmetic when the float value lands inside the margin, so the lists are the fp64
// lists exactly.
//
// Load balance: the warp-per-leaf kernels hand a leaf over to a heavy-leaf kernel when its
// lists outgrow the warp's shared memory (density: the gather list or a particle's
// compact list; forces: the near or direct-sum list).  The heavy-leaf kernels give such a
// leaf a whole block — density: one warp per particle, each iteration walking the tree
// for the particle's own 2h box; forces: 8 warps sharing the leaf's lists round-robin.
#include "gsph_state.cuh"
#include "gsph_walk.cuh"
#include "kernels.cuh"
#include "mixed_state.cuh"
#include "batch.cuh"
#include "stars.cuh"

namespace gsph {

namespace {

constexpr float kMargin = 6.103515625e-05f;   // 2^-14 relative
constexpr int kNodeBits = 25;
constexpr int kNoShift = 13;

// A leaf of the force walk's near and direct-sum lists as one word: its first slot and
// particle count, (first << 5) | (n - 1), taken from the walk's own cell load, so that the
// list consumers read no cell arrays (leaves hold 1..32 particles; the mixed form takes up
// to 2^27 particles).
constexpr int kLeafCountBits = 5;
constexpr int kMixedMaxParticles = 1 << (32 - kLeafCountBits);
__device__ __forceinline__ unsigned pack_leaf(int first, int n) {
  return ((unsigned) first << kLeafCountBits) | (unsigned) (n - 1);
}
__device__ __forceinline__ int leaf_first(unsigned w) { return (int) (w >> kLeafCountBits); }
__device__ __forceinline__ int leaf_count(unsigned w) { return (int) (w & ((1u << kLeafCountBits) - 1u)) + 1; }

// The w lane of a cell's float bounding-box maximum: (cell_first << 5) | level (at most 23
// levels), so that a walk decision's box loads also give the list word of an emitted leaf.
constexpr int kLevelBits = 5;
__device__ __forceinline__ int box_level(float w) { return __float_as_int(w) & ((1 << kLevelBits) - 1); }
__device__ __forceinline__ int box_first(float w) { return (int) ((unsigned) __float_as_int(w) >> kLevelBits); }

// ---- preparation --------------------------------------------------------------------
__device__ __forceinline__ void split2(double v, float& hi, float& lo) {
  hi = __double2float_rn(v);
  lo = __double2float_rn(v - (double) hi);
}

__global__ void k_prep_build_particles(Particles p, MixedParticles mp) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < p.n; s += gridDim.x * blockDim.x) {
    float xh, xl, yh, yl, zh, zl;
    split2(p.x[s], xh, xl);
    split2(p.y[s], yh, yl);
    split2(p.z[s], zh, zl);
    mp.pos_hi[s] = make_float4(xh, yh, zh, __double2float_rn(p.m[s]));
    mp.pos_lo[s] = make_float4(xl, yl, zl, 0.0f);
  }
}

__global__ void k_prep_build_cells(Tree t, MixedCells mc) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < t.ncell; c += gridDim.x * blockDim.x) {
    const CellGeom g = t.geom[c];
    const CellMoment m = t.mom[c];
    const CellBox b = t.bb[c];
    float h[3], l[3];
    for (int k = 0; k < 3; k++) split2(g.rcell[k], h[k], l[k]);
    mc.geo_hi[c] = make_float4(h[0], h[1], h[2], __double2float_rn(g.rmax));
    mc.geo_lo[c] = make_float4(l[0], l[1], l[2], __double2float_rn(g.hmax));
    mc.meta[c] = make_float4(__double2float_rn(g.cdistsqd), __int_as_float(t.cell_n[c]),
                             __int_as_float((int) t.cell_level[c]), __int_as_float(t.cell_first[c]));
    for (int k = 0; k < 3; k++) split2(m.r[k], h[k], l[k]);
    mc.com_hi[c] = make_float4(h[0], h[1], h[2], __double2float_rn(m.m));
    mc.com_lo[c] = make_float4(l[0], l[1], l[2], __double2float_rn(m.q[4]));
    mc.quad[c] = make_float4(__double2float_rn(m.q[0]), __double2float_rn(m.q[1]), __double2float_rn(m.q[2]),
                             __double2float_rn(m.q[3]));
    mc.bbmin[c] = make_float4(__double2float_rd(b.bbmin[0]), __double2float_rd(b.bbmin[1]),
                              __double2float_rd(b.bbmin[2]), __int_as_float(t.cell_n[c]));
    mc.bbmax[c] = make_float4(__double2float_ru(b.bbmax[0]), __double2float_ru(b.bbmax[1]),
                              __double2float_ru(b.bbmax[2]),
                              __int_as_float((int) (((unsigned) t.cell_first[c] << kLevelBits) | t.cell_level[c])));
  }
}

// The float quotients 1/h, 1/rho and P Omega^-1 / rho^2 are formed from the float values
// (correctly rounded reciprocals; within an ulp or two of the rounded fp64 quotients): fp64
// divisions would hold GB300's fp64 pipe for 64 cycles a warp instruction each.
__global__ void k_prep_hydro_particles(Particles p, MixedParticles mp) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < p.n; s += gridDim.x * blockDim.x) {
    const float hf = __double2float_rn(p.h[s]), rf = __double2float_rn(p.rho[s]);
    mp.vel[s] = make_float4(__double2float_rn(p.vx[s]), __double2float_rn(p.vy[s]), __double2float_rn(p.vz[s]), hf);
    const float ir = __frcp_rn(rf);
    const float fac = __double2float_rn(p.pressure[s]) * __double2float_rn(p.invomega[s]) * ir * ir;
    mp.hyd[s] = make_float4(__frcp_rn(hf), fac, ir, __double2float_rn(p.sound[s]));
    mp.aux[s] = make_float4(__double2float_rn(p.hfactor[s]), __double2float_rn(p.zeta[s]),
                            __double2float_rn(p.hrangesqd[s]), 0.0f);
    mp.pos_lo[s].w = __double2float_rn(p.hrangesqd[s]);   // the neighbour test's candidate load
  }
}

__global__ void k_prep_hydro_cells(Tree t, MixedCells mc) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < t.ncell; c += gridDim.x * blockDim.x) {
    const CellGeom g = t.geom[c];
    const CellBox hb = t.hbox[c];
    float4 lo = mc.geo_lo[c];
    lo.w = __double2float_rn(g.hmax);
    mc.geo_lo[c] = lo;
    mc.hbmin[c] = make_float4(__double2float_rd(hb.bbmin[0]), __double2float_rd(hb.bbmin[1]),
                              __double2float_rd(hb.bbmin[2]), 0.0f);
    mc.hbmax[c] = make_float4(__double2float_ru(hb.bbmax[0]), __double2float_ru(hb.bbmax[1]),
                              __double2float_ru(hb.bbmax[2]), 0.0f);
  }
}

// ---- helpers ------------------------------------------------------------------------------
template <int LPG>
__device__ __forceinline__ double gsum_d(double v) {
#pragma unroll
  for (int o = 1; o < LPG; o <<= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}
template <int LPG>
__device__ __forceinline__ float gsum_f(float v) {
#pragma unroll
  for (int o = 1; o < LPG; o <<= 1) v = __fadd_rn(v, __shfl_xor_sync(kFull, v, o));
  return v;
}
// The same sums over groups of a run-time width (a power of two, uniform over the warp).
__device__ __forceinline__ double gsum_d(double v, int lpg) {
  for (int o = 1; o < lpg; o <<= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}
__device__ __forceinline__ float gsum_f(float v, int lpg) {
  for (int o = 1; o < lpg; o <<= 1) v = __fadd_rn(v, __shfl_xor_sync(kFull, v, o));
  return v;
}

__device__ __forceinline__ float fsqrt_pos(float x) { return x > 0.0f ? x * rsqrtf(x) : 0.0f; }

// Index of the k-th set bit of m (k < popc(m)).
__device__ __forceinline__ int nth_bit(unsigned m, int k) {
  for (int i = 0; i < k; i++) m &= m - 1u;
  return __ffs(m) - 1;
}

__device__ __forceinline__ bool fbox_overlap(const float* amin, const float* amax, float4 bmin, float4 bmax) {
  if (amin[0] > bmax.x || bmin.x > amax[0]) return false;
  if (amin[1] > bmax.y || bmin.y > amax[1]) return false;
  if (amin[2] > bmax.z || bmin.z > amax[2]) return false;
  return true;
}

__device__ __forceinline__ double shift_of(int code, int k, const SphParams& prm) {
  const int d = (k == 0 ? code % 3 : (k == 1 ? (code / 3) % 3 : code / 9)) - 1;
  return d == 0 ? 0.0 : (d > 0 ? prm.boxsize[k] : -prm.boxsize[k]);
}

// ==========================================================================================
// Density / h solve, mixed form.
//
// One cell's solve by one warp (WARPS = 1), shared by the single-simulation and the batch
// kernels.  The template also carries a block-wide form (WARPS warps share one cell, its
// candidate leaves dealt round-robin, per-iteration sums combined in warp order in shared
// memory) that no kernel instantiates at present: leaves too large for one warp go to the
// per-particle heavy-leaf kernel instead.
// ==========================================================================================
constexpr int kDensStack = 1024;
constexpr int kDensListNormal = 256;    // leaves a warp handles alone
constexpr int kMaxAttempts = 256;

struct DensSmem {
  float part[8][8][3];   // [warp][group][rho, omega, zeta]
  int flag[8];
};

// One step of GradhSph::ComputeH's h iteration (src/GradhSph/GradhSph.cpp:206-254) from
// the kernel sums of the current h (drho = sum m W, dom = sum m h^-1 Womega, dze = sum m
// Wzeta, before the h^-3 / h^-2 factors): the convergence test against h_fac (m /
// rho)^(1/3), then a fixed-point step (iterations < 30) or bisection (up to 150).
// h_fac (m/rho)^(1/3) = h_fac h w^(-1/3) with w = rho h^3 / m: a float reciprocal cube
// root refined by one fp64 Newton step (relative error ~1e-14).  Sets done when the
// particle has finished (converged, left the bracket, aborted with h > hmax_list, or failed
// to converge).  rho, om and zeta (the density and its terms at this h) are formed only
// when they are used: on finishing and in the bisection test; rho > 0 is tested as drho > 0
// (h^-3 > 0).  GB300 runs fp64 at 1/64 of the fp32 rate, so the update keeps to the fp64
// operations the test and the h sequence need.
__device__ __forceinline__ void h_update(double drho, double dom, double dze, double inv_m, double inv_hfac,
                                         double hmax_list, const SphParams& prm, int iteration,
                                         double& hi, double& invh, double& h_lower, double& h_upper,
                                         double& hrho_last, double& rho, double& om, double& zeta, double& mloc,
                                         bool& done, bool& abort_cell, bool& fail) {
  const double invh0 = invh;
  auto density = [&]() {
    const double isq = invh0 * invh0, hfac3 = invh0 * isq;
    rho = drho * hfac3;
    om = dom * hfac3;
    zeta = dze * isq;
  };
  const double w = drho * inv_m;
  double r = (double) rcbrtf((float) w);
  r = r * (4.0 / 3.0 - (w * (1.0 / 3.0)) * (r * r * r));
  const double hrho = prm.h_fac * hi * r;
  hrho_last = hrho;
  // h_lower is 0 until the bisection starts (iteration 31)
  if (drho > 0.0 && (iteration <= 30 || hi > h_lower) && fabs(hi - hrho) * invh < prm.h_converge) {
    density();
    done = true;
    return;
  }
  if (iteration < 30) {
    invh = invh * (w * r * r) * inv_hfac;   // 1 / hrho
    hi = hrho;
  } else {
    if (iteration == 30) hi = 0.5 * (h_lower + h_upper);
    else if (iteration < 150) {
      density();
      if (rho < kSmall || hi > hrho) h_upper = hi; else h_lower = hi;
      hi = 0.5 * (h_lower + h_upper);
    } else {
      density();
      fail = true;
      done = true;
      return;
    }
    invh = 1.0 / hi;
  }
  mloc = fmax(mloc, hi);
  if (hi > hmax_list) { abort_cell = true; done = true; }
  else if (!(hi > h_lower && hi < h_upper)) done = true;
  if (done) density();
}

// Final per-particle results of the h solve (GradhSph.cpp:262-317): h, rho, hfactor,
// hrangesqd, invomega, zeta (with the SPH-star term), the EOS quantities.
// The derived quantities in single precision (the form's h and rho carry float accuracy),
// stored as fp64; hrangesqd keeps the fp64 product, which the exact membership checks use.
__device__ __forceinline__ void finish_density(const Particles& p, const SphParams& prm, int slot, double hfin,
                                               double rho_out, double om_out, double zeta_out, double star_zeta) {
  const float hf = (float) hfin, rf = (float) rho_out;
  const float invh = __frcp_rn(hf);
  const float ih2 = invh * invh;
  p.h[slot] = hfin;
  p.rho[slot] = rho_out;
  p.hfactor[slot] = (double) (ih2 * ih2);
  p.hrangesqd[slot] = __dmul_rn(__dmul_rn(kKernRangeSqd, hfin), hfin);
  p.div_v[slot] = 0.0;
  const float drho = -(1.0f / 3.0f) * hf * __frcp_rn(rf);
  const float io = __frcp_rn(1.0f - drho * (float) om_out);
  p.invomega[slot] = (double) io;
  p.zeta[slot] = (double) (drho * (float) (zeta_out + star_zeta) * io);
  double u = p.u[slot];
  if (prm.eos == 1) { u = prm.u_iso; p.u[slot] = u; }
  const float gm1 = (float) (prm.gamma_eos - 1.0), uf = (float) u;
  p.sound[slot] = (double) (prm.eos == 1 ? sqrtf(gm1 * uf) : sqrtf((float) prm.gamma_eos * gm1 * uf));
  p.pressure[slot] = (double) (gm1 * rf * uf);
}

template <int LPG, int WARPS>
__device__ __forceinline__ bool density_cell(const Tree& t, const Particles& p, const MixedParticles& mp,
                                             const MixedCells& mc, const SphParams& prm, const DeviceCounters& cnt,
                                             int leaf, int* stack, int* list, int list_cap, float2* compact,
                                             int kcap, bool give_up, DensSmem* sm) {
  // WARPS > 1: the block's warps share the cell, each keeping every WARPS-th leaf of
  // the gather list; per-iteration sums are added across warps in warp order.
  const int lane = threadIdx.x & 31;
  const int wib = WARPS > 1 ? (threadIdx.x >> 5) : 0;
  const int g = lane / LPG, sl = lane % LPG;
  const int c = t.leaf_cell[leaf];
  const int first = t.cell_first[c], ncell = t.cell_n[c];
  const bool mine = g < ncell && is_active(p, first + g);
  if (!__any_sync(kFull, mine)) return true;   // no active particle in this leaf
  const int slot = first + (g < ncell ? g : 0);
  // active particles of the leaf, one bit each (warp-uniform)
  constexpr int G = 32 / LPG;
  unsigned amask = 0;
  {
    const unsigned gm = __ballot_sync(kFull, mine && sl == 0);
#pragma unroll
    for (int q = 0; q < G; q++)
      if ((gm >> (q * LPG)) & 1u) amask |= 1u << q;
  }
  const int nact = __popc(amask);
  // Lanes of the h iteration.  When every active particle's compact list fits (leaves
  // that do not are handed over, give_up), the active particles share the warp evenly —
  // 32 / p lanes each, p the power of two at or above their count — instead of LPG lanes
  // per particle, so the lanes of inactive particles (block timesteps) do not idle.
  const bool remap = give_up && WARPS == 1;
  int it_g = g, it_sl = sl, it_L = LPG;
  if (remap) {
    int p2 = 1;
    while (p2 < nact) p2 <<= 1;
    it_L = 32 / p2;
    const int k = lane / it_L;
    it_sl = lane % it_L;
    it_g = k < nact ? nth_bit(amask, k) : -1;
  }
  const bool it_mine = remap ? it_g >= 0 : mine;
  const int it_slot = first + (it_g >= 0 && it_g < ncell ? it_g : 0);
  const double it_m = p.m[it_slot], it_h0 = p.h[it_slot];
  const double it_inv_m = it_sl == 0 ? 1.0 / it_m : 0.0;
  const double inv_hfac = it_sl == 0 ? 1.0 / prm.h_fac : 0.0;
  const float4 pih = mp.pos_hi[slot], pil = mp.pos_lo[slot];
  const double xi = p.x[slot], yi = p.y[slot], zi = p.z[slot];
  const CellBox bb = t.bb[c];
  const double hmax0 = t.geom[c].hmax;
  unsigned long long pairs = 0;
  bool fail = false, stack_ok = true;
  double mcheck = 0.0;
  double h_out = it_h0, rho_out = 0.0, om_out = 0.0, zeta_out = 0.0;

  // returns 1 if the cell aborts (some h > hmax_list), 2 if the warp gives up (gather or
  // compact list too long for a warp on its own; only when give_up), 0 when solved
  auto attempt = [&](double hmax_list) -> int {
    const double hr = __dmul_rn(kKernRange, hmax_list);
    double gmin[3], gmax[3];
    for (int k = 0; k < 3; k++) { gmin[k] = __dsub_rn(bb.bbmin[k], hr); gmax[k] = __dadd_rn(bb.bbmax[k], hr); }
    int nsh[3] = {1, 1, 1}, sh[3][3];
    for (int k = 0; k < 3; k++) {
      sh[k][0] = 1;
      if (prm.periodic) {
        if (gmax[k] > prm.boxmax[k]) sh[k][nsh[k]++] = 2;
        if (gmin[k] < prm.boxmin[k]) sh[k][nsh[k]++] = 0;
      }
    }
    WarpLists L{list, list, list, 0, 0, 0, list_cap};
    L.mod = WARPS; L.sel = wib;
    bool overflow = false;
    auto walk_all = [&](auto&& flush) {
      L.emitted_a = 0;
      for (int a0 = 0; a0 < nsh[0]; a0++)
        for (int a1 = 0; a1 < nsh[1]; a1++)
          for (int a2 = 0; a2 < nsh[2]; a2++) {
            const int code = sh[0][a0] + 3 * sh[1][a1] + 9 * sh[2][a2];
            float bmin[3], bmax[3];
            for (int k = 0; k < 3; k++) {
              const double s = shift_of(code, k, prm);
              bmin[k] = __double2float_rd(gmin[k] - s);
              bmax[k] = __double2float_ru(gmax[k] - s);
            }
            // cell count, level and first slot ride in the float box's w lanes: two loads a
            // decision, and an emitted leaf's list word (open boxes: the leaf itself; periodic
            // boxes: node and image code, the slots read from the cell arrays)
            unsigned lw = 0;
            auto decide = [&](int node, int& level) -> int {
              const float4 b0 = mc.bbmin[node], b1 = mc.bbmax[node];
              level = box_level(b1.w);
              if (__float_as_int(b0.w) == 0) return kSkip;
              if (!fbox_overlap(bmin, bmax, b0, b1)) return kSkip;
              lw = pack_leaf(box_first(b1.w), __float_as_int(b0.w));
              return level == t.ltot ? kEmitA : kOpen;
            };
            auto tag = [&](int node, int) { return prm.periodic ? node | (code << kNodeBits) : (int) lw; };
            stack_ok = stack_ok && warp_walk_lv(0, t.ltot, stack, kDensStack, L, decide, tag, flush);
          }
    };
    walk_all([&]() { overflow = true; });
    if (give_up && __any_sync(kFull, overflow)) return 2;
    const int ncached = L.na;
    // a gather-list entry: the leaf's first slot and count, and the periodic image code
    auto entry = [&](int tagv, int& f, int& nn, int& code) {
      if (prm.periodic) {
        const int node = tagv & ((1 << kNodeBits) - 1);
        code = tagv >> kNodeBits;
        f = t.cell_first[node];
        nn = t.cell_n[node];
      } else {
        f = leaf_first((unsigned) tagv);
        nn = leaf_count((unsigned) tagv);
        code = kNoShift;
      }
    };

    // The candidate's separation from this particle in float (false: that periodic
    // image does not exist, ghost semantics as in the fp64 form).
    auto cand = [&](int j, int code, float& d2, float& mj) -> bool {
      float dx, dy, dz;
      const float4 pjh = mp.pos_hi[j];
      mj = pjh.w;
      if (code == kNoShift) {
        const float4 pjl = mp.pos_lo[j];
        dx = (pjh.x - pih.x) + (pjl.x - pil.x);
        dy = (pjh.y - pih.y) + (pjl.y - pil.y);
        dz = (pjh.z - pih.z) + (pjl.z - pil.z);
      } else {
        const double sx = shift_of(code, 0, prm), sy = shift_of(code, 1, prm), sz = shift_of(code, 2, prm);
        const double xj = p.x[j], yj = p.y[j], zj = p.z[j];
        const double lim = __dmul_rn(kGhostRange * kKernRange, p.h0[j]);
        bool ok = true;
        if (sx > 0.0) ok = ok && (xj < __dadd_rn(prm.boxmin[0], lim));
        if (sx < 0.0) ok = ok && (xj > __dsub_rn(prm.boxmax[0], lim));
        if (sy > 0.0) ok = ok && (yj < __dadd_rn(prm.boxmin[1], lim));
        if (sy < 0.0) ok = ok && (yj > __dsub_rn(prm.boxmax[1], lim));
        if (sz > 0.0) ok = ok && (zj < __dadd_rn(prm.boxmin[2], lim));
        if (sz < 0.0) ok = ok && (zj > __dsub_rn(prm.boxmax[2], lim));
        if (!ok) return false;
        dx = (float) (__dadd_rn(xj, sx) - xi);
        dy = (float) (__dadd_rn(yj, sy) - yi);
        dz = (float) (__dadd_rn(zj, sz) - zi);
      }
      d2 = dx * dx + dy * dy + dz * dz;
      return true;
    };

    // The candidate's position as a hi + lo float pair (its periodic image for code !=
    // kNoShift); false: that image does not exist.  ch.w = mass.
    auto cand_pos = [&](int j, int code, float4& ch, float4& cl) -> bool {
      if (code == kNoShift) { ch = mp.pos_hi[j]; cl = mp.pos_lo[j]; return true; }
      const double sx = shift_of(code, 0, prm), sy = shift_of(code, 1, prm), sz = shift_of(code, 2, prm);
      const double xj = p.x[j], yj = p.y[j], zj = p.z[j];
      const double lim = __dmul_rn(kGhostRange * kKernRange, p.h0[j]);
      bool ok = true;
      if (sx > 0.0) ok = ok && (xj < __dadd_rn(prm.boxmin[0], lim));
      if (sx < 0.0) ok = ok && (xj > __dsub_rn(prm.boxmax[0], lim));
      if (sy > 0.0) ok = ok && (yj < __dadd_rn(prm.boxmin[1], lim));
      if (sy < 0.0) ok = ok && (yj > __dsub_rn(prm.boxmax[1], lim));
      if (sz > 0.0) ok = ok && (zj < __dadd_rn(prm.boxmin[2], lim));
      if (sz < 0.0) ok = ok && (zj > __dsub_rn(prm.boxmax[2], lim));
      if (!ok) return false;
      const double X = __dadd_rn(xj, sx), Y = __dadd_rn(yj, sy), Z = __dadd_rn(zj, sz);
      ch = make_float4((float) X, (float) Y, (float) Z, mp.pos_hi[j].w);
      cl = make_float4((float) (X - (double) ch.x), (float) (Y - (double) ch.y), (float) (Z - (double) ch.z), 0.f);
      return true;
    };

    // Per-particle compact lists of (d^2, m) for the pairs inside 2 hmax_list (the
    // reference's own pre-filter, GradhSphTree.cpp:205-219), built once per attempt; a
    // particle whose list does not fit loops over the candidates instead.  The build runs
    // one candidate per lane (LPG leaves of up to 32/LPG particles per round, coalesced
    // loads) against every particle of the cell, eight at a time from registers.
    const unsigned ltm = (1u << lane) - 1u;
    int ccount = 0;
    const float lim2 = (float) (kKernRangeSqd * hmax_list * hmax_list) * (1.0f + kMargin);
    if (!overflow) {
      const int ntgt = nact;   // the active particles only: the others solve nothing
      // positions relative to the leaf centre (hi + lo pairs): a few float ulps of the
      // separation, three registers a target
      const float4 lch = mc.geo_hi[c], lcl = mc.geo_lo[c];
      for (int gc = 0; gc < ntgt; gc += 8) {
        float tx[8], ty[8], tz[8];
        int tc[8], tgi[8];
#pragma unroll
        for (int u = 0; u < 8; u++) {
          const int tg = nth_bit(amask, gc + u < ntgt ? gc + u : ntgt - 1);
          tgi[u] = tg;
          const float4 h = mp.pos_hi[first + tg], l = mp.pos_lo[first + tg];
          tx[u] = (h.x - lch.x) + (l.x - lcl.x);
          ty[u] = (h.y - lch.y) + (l.y - lcl.y);
          tz[u] = (h.z - lch.z) + (l.z - lcl.z);
          tc[u] = 0;
        }
        for (int e0 = 0; e0 < ncached; e0 += LPG) {
          const int e = e0 + lane / G, q = lane % G;
          bool valid = false;
          float4 ch = make_float4(0.f, 0.f, 0.f, 0.f), cl = ch;
          if (e < ncached) {
            int f, nn, code;
            entry(list[e], f, nn, code);
            if (q < nn) valid = cand_pos(f + q, code, ch, cl);
          }
          const float cx = (ch.x - lch.x) + (cl.x - lcl.x);
          const float cy = (ch.y - lch.y) + (cl.y - lcl.y);
          const float cz = (ch.z - lch.z) + (cl.z - lcl.z);
#pragma unroll
          for (int u = 0; u < 8; u++) {
            if (gc + u >= ntgt) break;
            const float dx = cx - tx[u];
            const float dy = cy - ty[u];
            const float dz = cz - tz[u];
            const float d2 = dx * dx + dy * dy + dz * dz;
            const bool keep = valid && d2 <= lim2;
            const unsigned b = __ballot_sync(kFull, keep);
            if (keep) {
              const int pos = tc[u] + __popc(b & ltm);
              if (pos < kcap) compact[tgi[u] * kcap + pos] = make_float2(d2, ch.w);
            }
            tc[u] += __popc(b);
          }
        }
#pragma unroll
        for (int u = 0; u < 8; u++)
          if (gc + u < ntgt && tgi[u] == g) ccount = tc[u];
      }
    }
    // A particle whose compact list does not fit would rescan every candidate in every
    // iteration, and its warp with it (such leaves took 5-10x the mean): hand the leaf to
    // the heavy-leaf kernel instead.
    if (give_up && __any_sync(kFull, mine && !overflow && ccount > kcap)) return 2;
    // the iteration lane's particle: its compact list and count (held by its group's lanes)
    const int cg = it_g >= 0 ? it_g : 0;
    const int ccount_it = __shfl_sync(kFull, ccount, cg * LPG);
    float2* clist = compact + cg * kcap;
    const bool use_compact = remap || (!overflow && ccount <= kcap);

    // The iteration state (h, its bracket, the h(rho) target) and the convergence test are
    // fp64, as in the reference (GradhSph.cpp:206-254); the kernel sums are float.  The
    // fp64 update runs on the first lane of the particle's group only (an fp64 instruction
    // occupies GB300's fp64 pipe for every active lane), which passes the float 1/h, 1/h^2
    // and the done flag to the group's other lanes.
    const bool lead = it_sl == 0;
    const int lead_lane = lane - it_sl;
    double hi = it_h0, h_lower = 0.0, h_upper = hmax_list;
    double invh = lead ? 1.0 / hi : 0.0, hrho_last = hi;
    double rho = 0.0, om = 0.0, zeta = 0.0;
    int iteration = 0;
    bool done = !it_mine, abort_cell = false;
    double mloc = 0.0;
    for (;;) {
      bool any_active = __any_sync(kFull, !done);
      if (WARPS > 1) any_active = __syncthreads_or(any_active);
      if (!any_active) break;
      iteration++;
      float invh_f = 0.0f, invhsqd_f = 0.0f;
      if (lead) {
        invh_f = (float) invh;
        invhsqd_f = (float) (invh * invh);
      }
      invh_f = __shfl_sync(kFull, invh_f, lead_lane);
      invhsqd_f = __shfl_sync(kFull, invhsqd_f, lead_lane);
      float srho = 0.0f, som = 0.0f, sze = 0.0f;
      float crho = 0.0f, com = 0.0f, cze = 0.0f;   // compensation terms (compensated sums)
      const bool comp = prm.compensated != 0;
      auto add = [&](float d2, float mj) {
        const float ssqd = d2 * invhsqd_f;
        if (ssqd < 4.0f) {
          const float s = fsqrt_pos(ssqd);
          float w0, wom, wze;   // s < 2 here
          m4f_w0_omega_zeta(s, w0, wom, wze);
          if (comp) {
            kahan_add(srho, crho, mj * w0);
            kahan_add(som, com, (mj * invh_f) * wom);
            kahan_add(sze, cze, mj * wze);
          } else {
            srho = fmaf(mj, w0, srho);
            som = fmaf(mj * invh_f, wom, som);
            sze = fmaf(mj, wze, sze);
          }
          pairs++;
        }
      };
      auto consume = [&](int count) {
        if (done) return;
        for (int e = 0; e < count; e++) {
          int f, nn, code;
          entry(list[e], f, nn, code);
          for (int q = sl; q < nn; q += LPG) {
            float d2, mj;
            if (cand(f + q, code, d2, mj)) add(d2, mj);
          }
        }
      };
      if (use_compact) {
        if (!done) for (int e = it_sl; e < ccount_it; e += it_L) { const float2 v = clist[e]; add(v.x, v.y); }
      } else if (!overflow) {
        consume(ncached);
      } else {
        L = WarpLists{list, list, list, 0, 0, 0, list_cap};
        L.mod = WARPS; L.sel = wib;
        walk_all([&]() { consume(L.na); });
        consume(L.na);
      }
      double drho, dom, dze;
      if (comp) {   // the lanes' compensated partials combined in fp64
        drho = (double) srho - (double) crho;
        dom = (double) som - (double) com;
        dze = (double) sze - (double) cze;
        for (int o = 1; o < it_L; o <<= 1) {
          drho += __shfl_xor_sync(kFull, drho, o);
          dom += __shfl_xor_sync(kFull, dom, o);
          dze += __shfl_xor_sync(kFull, dze, o);
        }
      } else {
        for (int o = 1; o < it_L; o <<= 1) {
          srho += __shfl_xor_sync(kFull, srho, o);
          som += __shfl_xor_sync(kFull, som, o);
          sze += __shfl_xor_sync(kFull, sze, o);
        }
        drho = srho; dom = som; dze = sze;
      }
      if (WARPS > 1) {
        if (sl == 0) {
          sm->part[wib][g][0] = (float) drho; sm->part[wib][g][1] = (float) dom; sm->part[wib][g][2] = (float) dze;
        }
        __syncthreads();
        float fr = 0.0f, fo = 0.0f, fz = 0.0f;
        for (int w = 0; w < WARPS; w++) { fr += sm->part[w][g][0]; fo += sm->part[w][g][1]; fz += sm->part[w][g][2]; }
        drho = fr; dom = fo; dze = fz;
        __syncthreads();
      }
      if (!done && lead)
        h_update(drho, dom, dze, it_inv_m, inv_hfac, hmax_list, prm, iteration, hi,
                 invh, h_lower, h_upper, hrho_last, rho, om, zeta, mloc, done, abort_cell, fail);
      done = __shfl_sync(kFull, done, lead_lane);
    }
    double mw = mloc;
    for (int o = 16; o > 0; o >>= 1) mw = fmax(mw, __shfl_xor_sync(kFull, mw, o));
    bool any_abort = __any_sync(kFull, abort_cell);
    if (WARPS > 1) any_abort = __syncthreads_or(any_abort);
    mcheck = fmax(mcheck, mw);
    if (!any_abort && it_mine && lead) {
      h_out = fmax(hrho_last, h_lower);
      rho_out = rho; om_out = om; zeta_out = zeta;
    }
    if (!any_abort) h_out = __shfl_sync(kFull, h_out, lead_lane);   // the star term's lanes
    return any_abort ? 1 : 0;
  };

  // The reference's hmax sequence with the exact skip-ahead of density.cu.
  bool solved = false;
  double hk = __dmul_rn(1.05, hmax0);
  for (int a = 0; a < kMaxAttempts && !solved; a++) {
    const int r = attempt(hk);
    if (r == 2) return false;   // handed over to the heavy-leaf kernel
    if (r == 0) {
      solved = true;
    } else {
      int guard = 0;
      do { hk = __dmul_rn(1.05, hk); } while (hk < mcheck && ++guard < 100000);
    }
  }
  if (lane == 0 && !solved) atomicOr(cnt.status, (unsigned) kStatusRetryLimit);
  if (!stack_ok && lane == 0) atomicOr(cnt.status, (unsigned) kStatusStackOverflow);
  if (__any_sync(kFull, fail) && lane == 0) atomicOr(cnt.status, (unsigned) kStatusHNotConverged);
  unsigned long long tot = pairs;
  for (int o = 16; o > 0; o >>= 1) tot += __shfl_xor_sync(kFull, tot, o);
  if (lane == 0) atomicAdd(cnt.density_pairs, tot);
  // the SPH-star zeta term, the particle's LPG lanes sharing the stars
  float zs = 0.0f;
  if (prm.stars.n) {
    if (it_mine) zs = star_zeta_part_f(prm.stars, mp.pos_hi[it_slot], mp.pos_lo[it_slot], (float) h_out, it_sl, it_L);
    for (int o = 1; o < it_L; o <<= 1) zs += __shfl_xor_sync(kFull, zs, o);
  }
  if (it_mine && it_sl == 0 && wib == 0) finish_density(p, prm, it_slot, h_out, rho_out, om_out, zeta_out, (double) zs);
  return true;
}


// Heavy leaves: one block per leaf, one warp per particle (particles g, g + 8, ... of the
// leaf).  Instead of scanning the leaf's whole gather list every iteration, each
// iteration walks the tree for the particle's own search box r_i +- 2 h_i: every pair
// inside the kernel support of the current h is inside the leaf's gather box (h stays
// below hmax_list while the attempt runs), so the sums take the same pairs as the
// gather-list form.  The cell-level attempt protocol (abort when some h exceeds
// hmax_list, exact skip-ahead of the 1.05 sequence) is kept across the block.
constexpr int kPPStack = 1024;
constexpr int kPPList = 256;

struct PPShared {
  int stack[8][kPPStack];
  int list[8][kPPList];
  double h0[32];
  double mloc[8];
};

// One heavy leaf, solved by the whole block (256 threads); interaction counts and status
// go to cnt when the leaf is done.
template <int LPG>
__device__ __forceinline__ void density_pp_leaf(const Tree& t, const Particles& p, const MixedParticles& mp,
                                                const MixedCells& mc, const SphParams& prm,
                                                const DeviceCounters& cnt, int leaf, PPShared& sm) {
  constexpr int G = 32 / LPG;   // lanes per leaf when scanning emitted leaves
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
      const float4 pih = mp.pos_hi[slot], pil = mp.pos_lo[slot];
      const double xi = p.x[slot], yi = p.y[slot], zi = p.z[slot], mi = p.m[slot];
      // the fp64 update on lane 0, which passes h, the float 1/h, 1/h^2 and done to the warp
      double hi = sm.h0[g], h_lower = 0.0, h_upper = hk;
      double invh = lane == 0 ? 1.0 / hi : 0.0, hrho_last = hi;
      const double inv_m = lane == 0 ? 1.0 / mi : 0.0, inv_hfac = lane == 0 ? 1.0 / prm.h_fac : 0.0;
      double rho = 0.0, om = 0.0, zeta = 0.0;
      bool done = false, abort_cell = false;
      int iteration = 0;
      while (!done) {
        iteration++;
        float invh_f = 0.0f, invhsqd_f = 0.0f;
        if (lane == 0) {
          invh_f = (float) invh;
          invhsqd_f = (float) (invh * invh);
        }
        invh_f = __shfl_sync(kFull, invh_f, 0);
        invhsqd_f = __shfl_sync(kFull, invhsqd_f, 0);
        float srho = 0.0f, som = 0.0f, sze = 0.0f;
        // the particle's search box, rounded outwards, and its periodic images
        const double rr = __dmul_rn(kKernRange * (1.0 + 1.0 / 1024.0), hi);
        double gmin[3] = {xi - rr, yi - rr, zi - rr}, gmax[3] = {xi + rr, yi + rr, zi + rr};
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
            float dx, dy, dz, mj;
            if (code == kNoShift) {
              const float4 pjh = mp.pos_hi[j], pjl = mp.pos_lo[j];
              mj = pjh.w;
              dx = (pjh.x - pih.x) + (pjl.x - pil.x);
              dy = (pjh.y - pih.y) + (pjl.y - pil.y);
              dz = (pjh.z - pih.z) + (pjl.z - pil.z);
            } else {
              const double sx = shift_of(code, 0, prm), sy = shift_of(code, 1, prm), sz = shift_of(code, 2, prm);
              const double xj = p.x[j], yj = p.y[j], zj = p.z[j];
              const double lim = __dmul_rn(kGhostRange * kKernRange, p.h0[j]);
              bool ok = true;
              if (sx > 0.0) ok = ok && (xj < __dadd_rn(prm.boxmin[0], lim));
              if (sx < 0.0) ok = ok && (xj > __dsub_rn(prm.boxmax[0], lim));
              if (sy > 0.0) ok = ok && (yj < __dadd_rn(prm.boxmin[1], lim));
              if (sy < 0.0) ok = ok && (yj > __dsub_rn(prm.boxmax[1], lim));
              if (sz > 0.0) ok = ok && (zj < __dadd_rn(prm.boxmin[2], lim));
              if (sz < 0.0) ok = ok && (zj > __dsub_rn(prm.boxmax[2], lim));
              if (!ok) continue;
              mj = mp.pos_hi[j].w;
              dx = (float) (__dadd_rn(xj, sx) - xi);
              dy = (float) (__dadd_rn(yj, sy) - yi);
              dz = (float) (__dadd_rn(zj, sz) - zi);
            }
            const float ssqd = (dx * dx + dy * dy + dz * dz) * invhsqd_f;
            if (ssqd < 4.0f) {
              const float sv = fsqrt_pos(ssqd);
              float w0, wom, wze;   // sv < 2 here
              m4f_w0_omega_zeta(sv, w0, wom, wze);
              srho = fmaf(mj, w0, srho);
              som = fmaf(mj * invh_f, wom, som);
              sze = fmaf(mj, wze, sze);
              pairs++;
            }
          }
          __syncwarp();
        };
        for (int a0 = 0; a0 < nsh[0]; a0++)
          for (int a1 = 0; a1 < nsh[1]; a1++)
            for (int a2 = 0; a2 < nsh[2]; a2++) {
              const int code = sh[0][a0] + 3 * sh[1][a1] + 9 * sh[2][a2];
              float bmin[3], bmax[3];
              for (int q = 0; q < 3; q++) {
                const double sft = shift_of(code, q, prm);
                bmin[q] = __double2float_rd(gmin[q] - sft);
                bmax[q] = __double2float_ru(gmax[q] - sft);
              }
              auto decide = [&](int node, int& level) -> int {
                const float4 b0 = mc.bbmin[node], b1 = mc.bbmax[node];   // w: cell_n, first << 5 | level
                level = box_level(b1.w);
                if (__float_as_int(b0.w) == 0) return kSkip;
                if (!fbox_overlap(bmin, bmax, b0, b1)) return kSkip;
                return level == t.ltot ? kEmitA : kOpen;
              };
              auto tag = [&](int node, int) { return node | (code << kNodeBits); };
              stack_ok = warp_walk_lv(0, t.ltot, stack, kPPStack, L, decide, tag, consume) && stack_ok;
              consume();
              L.na = 0;
            }
        for (int o = 16; o > 0; o >>= 1) {
          srho += __shfl_xor_sync(kFull, srho, o);
          som += __shfl_xor_sync(kFull, som, o);
          sze += __shfl_xor_sync(kFull, sze, o);
        }
        if (lane == 0)
          h_update(srho, som, sze, inv_m, inv_hfac, hk, prm, iteration, hi, invh, h_lower, h_upper,
                   hrho_last, rho, om, zeta, mloc, done, abort_cell, fail);
        hi = __shfl_sync(kFull, hi, 0);
        done = __shfl_sync(kFull, done, 0);
        if (!stack_ok) done = true;
      }
      abort_cell = __shfl_sync(kFull, abort_cell, 0);
      abort_any = abort_any || abort_cell;
      // the SPH-star zeta term, the warp's lanes sharing the stars (h is warp-uniform here)
      float zs = 0.0f;
      if (prm.stars.n && !abort_cell) {
        const double hfin = __shfl_sync(kFull, fmax(hrho_last, h_lower), 0);
        zs = star_zeta_part_f(prm.stars, pih, pil, (float) hfin, lane, 32);
        for (int o = 16; o > 0; o >>= 1) zs += __shfl_xor_sync(kFull, zs, o);
      }
      if (!abort_cell && lane == 0)
        finish_density(p, prm, slot, fmax(hrho_last, h_lower), rho, om, zeta, (double) zs);
    }
    if (lane == 0) sm.mloc[wib] = mloc;
    abort_any = __syncthreads_or(abort_any);
    if (!abort_any) { solved = true; break; }
    double mc_ = 0.0;
    for (int w = 0; w < 8; w++) mc_ = fmax(mc_, sm.mloc[w]);
    __syncthreads();
    int guard = 0;
    do { hk = __dmul_rn(1.05, hk); } while (hk < mc_ && ++guard < 100000);
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
__global__ void __launch_bounds__(256, 2)
k_density_mixed_pp(Tree t, Particles p, MixedParticles mp, MixedCells mc, SphParams prm, DeviceCounters cnt,
                   HeavyList heavy) {
  __shared__ PPShared sm;
  const int nh = *heavy.count;
  for (int k = blockIdx.x; k < nh; k += gridDim.x)
    density_pp_leaf<LPG>(t, p, mp, mc, prm, cnt, heavy.leaves[k], sm);
}

constexpr int kDensWarps = 4;
constexpr int kCompactPerWarp = 1536;   // float2 entries shared by the particle groups of a batch warp
// The single-simulation h solve in two tiers of the same warp-per-leaf code: every leaf with
// compact lists of kCompactNormal entries a warp (13 KB of shared memory a warp: 16 warps an
// SM), the leaves whose lists overflow that with kCompactWide entries (17 KB: 13 warps an
// SM); leaves that overflow both go to the per-particle heavy-leaf kernel.  The wide tier
// has the batch kernel's capacity, so a leaf reaches the heavy-leaf kernel in a batch exactly
// when it does in a single step, and the two give the same sums bit for bit.
constexpr int kCompactNormal = 1024;
constexpr int kCompactWide = kCompactPerWarp;

// Per-particle compact list capacity of a warp with cap entries, also the stride between
// the lists of its particle groups: congruent to LPG modulo 16 so that the groups' reads
// of 8-byte entries (lane sl of group g reads entry sl + LPG k) fall in distinct
// shared-memory banks.
__host__ __device__ constexpr int compact_stride(int lpg, int cap) {
  return lpg >= 16 ? cap / (32 / lpg) : ((cap / (32 / lpg) - lpg) / 16) * 16 + lpg;
}

size_t dens_smem(int warps, int cap = kCompactPerWarp) {
  return (sizeof(float2) * cap + sizeof(int) * (kDensStack + kDensListNormal)) * warps;
}

// One warp per block, one leaf per warp: a block's slot frees as soon as its leaf is
// done (leaf costs vary by an order of magnitude, and warps of a larger block would wait
// for the slowest).  At most 128 registers a thread, so that shared memory decides the
// warps an SM: 16 with kCompactNormal lists.  list == nullptr: leaf = block index (every
// leaf); otherwise the leaves list[0 .. *list_count) in a block-strided loop.  Leaves whose
// compact lists overflow cap entries go to out.
template <int LPG>
__global__ void __launch_bounds__(32, 16)
k_density_mixed(Tree t, Particles p, MixedParticles mp, MixedCells mc, SphParams prm, DeviceCounters cnt,
                HeavyList out, const int* list, const int* list_count, int cap) {
  extern __shared__ float2 s_dyn2[];
  float2* s_compact = s_dyn2;
  int* s_stack = reinterpret_cast<int*>(s_dyn2 + cap);
  int* s_list = s_stack + kDensStack;
  const int kcap = compact_stride(LPG, cap);
  // every leaf: this block's leaf only (the grid covers the leaves); a list: block-strided
  const int nl = list ? *list_count : min(t.nleaf, (int) blockIdx.x + 1);
  for (int k = blockIdx.x; k < nl; k += gridDim.x) {
    const int leaf = list ? list[k] : k;
    const bool ok = density_cell<LPG, 1>(t, p, mp, mc, prm, cnt, leaf, s_stack, s_list,
                                         tuned_depth(prm.gather_depth, 64, kDensListNormal), s_compact, kcap, true,
                                         nullptr);
    if (!ok && (threadIdx.x & 31) == 0) {
      const int q = atomicAdd(out.count, 1);
      out.leaves[q] = leaf;
    }
  }
}


// ==========================================================================================
// Forces, mixed form.
// ==========================================================================================
struct AccF {
  float ah[3], ag[3], gpot, dudt, divv;
  float cg[4];   // compensation of ag[0..2] and gpot (compensated sums; zero otherwise)
};

// One gravity contribution: plain float sums, or compensated ones (prm.compensated).
#define GSPH_ADD_G(A, comp, vx, vy, vz, vp)                                                      \
  do {                                                                                           \
    if (comp) {                                                                                  \
      kahan_add((A).ag[0], (A).cg[0], vx); kahan_add((A).ag[1], (A).cg[1], vy);                  \
      kahan_add((A).ag[2], (A).cg[2], vz); kahan_add((A).gpot, (A).cg[3], vp);                   \
    } else {                                                                                     \
      (A).ag[0] += vx; (A).ag[1] += vy; (A).ag[2] += vz; (A).gpot += vp;                         \
    }                                                                                            \
  } while (0)

// The target's float mirrors; its fp64 position and hrangesqd, which only the rare exact
// membership re-tests need, are read from the particle arrays there (registers are what
// limits the force kernels' occupancy).
struct TargetF {
  float4 ph, pl, vel, hyd, aux;   // see MixedParticles
  int slot;
};

__device__ __forceinline__ void load_target_f(const Particles& p, const MixedParticles& mp, int s, TargetF& T) {
  (void) p;
  T.ph = mp.pos_hi[s]; T.pl = mp.pos_lo[s]; T.vel = mp.vel[s]; T.hyd = mp.hyd[s]; T.aux = mp.aux[s];
  T.slot = s;
}

// SPH neighbour (1), direct term (0): float test with margin, exact fp64 when ambiguous.
template <class Count>
__device__ __forceinline__ int sph_member(const Particles& p, const TargetF& T, int j, float d2, float hrsj,
                                          const SphParams& prm, Count& exact) {
  const float thr = fmaxf(T.aux.z, hrsj);
  if (d2 < thr * (1.0f - kMargin)) return 1;
  if (d2 > thr * (1.0f + kMargin)) return 0;
  exact++;
  const int i = T.slot;
  double dx = __dsub_rn(p.x[j], p.x[i]), dy = __dsub_rn(p.y[j], p.y[i]), dz = __dsub_rn(p.z[j], p.z[i]);
  if (prm.periodic) {
    // the reference's image: nearest to the leaf centre, then corrected about the particle
    // (forces.cu k_hydro_fp64); for leaf cells far smaller than the box both give the
    // nearest image of j about i
    double* dd[3] = {&dx, &dy, &dz};
    for (int k = 0; k < 3; k++) {
      if (*dd[k] > prm.boxhalf[k]) *dd[k] = __dsub_rn(*dd[k], prm.boxsize[k]);
      else if (*dd[k] < -prm.boxhalf[k]) *dd[k] = __dadd_rn(*dd[k], prm.boxsize[k]);
    }
  }
  const double drsqd = dot3_rn(dx, dy, dz);
  return (drsqd >= p.hrangesqd[i] && drsqd >= p.hrangesqd[j]) ? 0 : 1;
}

__device__ __forceinline__ float pair_pressure_f(const SphParams& prm, const TargetF& T, float wi, float wj,
                                                 float facj, float invrhoj, float soundj, float mj, float dvdr,
                                                 float& dudt) {
  float paux = T.hyd.y * wi + facj * wj;
  if (dvdr < 0.0f) {
    const float winvrho = 0.25f * (wi + wj) * (T.hyd.z + invrhoj);
    const float vsignal = T.hyd.w + soundj - prm.ab_visc_f * dvdr;
    const float av = prm.alpha_visc_f * vsignal * dvdr * winvrho;
    paux -= av;
    dudt -= 0.5f * mj * av * dvdr;
  }
  return paux;
}

__device__ __forceinline__ void hydro_pair_f(const SphParams& prm, const MixedParticles& mp, const TargetF& T, int j,
                                             float dx, float dy, float dz, float d2, float mj, AccF& A) {
  const float4 vj = mp.vel[j], hj = mp.hyd[j], xj = mp.aux[j];
  const float inv = d2 > 0.0f ? rsqrtf(d2) : 0.0f;
  const float drmag = d2 * inv;
  const float ux = dx * inv, uy = dy * inv, uz = dz * inv;
  const float wi = T.aux.x * m4f_w1(drmag * T.hyd.x);
  const float wj = xj.x * m4f_w1(drmag * hj.x);
  const float dvdr = (vj.x - T.vel.x) * ux + (vj.y - T.vel.y) * uy + (vj.z - T.vel.z) * uz;
  A.divv -= mj * dvdr * wi;
  const float paux = pair_pressure_f(prm, T, wi, wj, hj.y, hj.z, hj.w, mj, dvdr, A.dudt);
  A.ah[0] += mj * ux * paux; A.ah[1] += mj * uy * paux; A.ah[2] += mj * uz * paux;
}

__device__ __forceinline__ void hydro_grav_pair_f(const SphParams& prm, const TargetF& T, float4 vj, float4 hj,
                                                  float4 xj, float dx, float dy, float dz, float d2, float mj, AccF& A) {
  const float r2 = d2 + 1.0e-20f;
  const float invdrmag = rsqrtf(r2);
  const float drmag = r2 * invdrmag;
  const float ux = dx * invdrmag, uy = dy * invdrmag, uz = dz * invdrmag;
  const float dvdr = (vj.x - T.vel.x) * ux + (vj.y - T.vel.y) * uy + (vj.z - T.vel.z) * uz;
  const float si = drmag * T.hyd.x, sj = drmag * hj.x;
  // 1/s = h / |r|: the float h of each particle (vel.w) times the pair's rsqrt
  float w1i, wgi, wpi, w1j, wgj, wpj;
  m4f_w1_grav_pot(si, T.vel.w * invdrmag, w1i, wgi, wpi);
  m4f_w1_grav_pot(sj, vj.w * invdrmag, w1j, wgj, wpj);
  const float wi = T.aux.x * w1i;
  const float wj = xj.x * w1j;
  const float paux = pair_pressure_f(prm, T, wi, wj, hj.y, hj.z, hj.w, mj, dvdr, A.dudt);
  A.ah[0] += mj * ux * paux; A.ah[1] += mj * uy * paux; A.ah[2] += mj * uz * paux;
  const float pg = 0.5f * (T.hyd.x * T.hyd.x * wgi + T.aux.y * wi + hj.x * hj.x * wgj + xj.y * wj);
  GSPH_ADD_G(A, prm.compensated, mj * ux * pg, mj * uy * pg, mj * uz * pg, 0.5f * mj * (T.hyd.x * wpi + hj.x * wpj));
  A.divv -= mj * dvdr * wi;
}

__device__ __forceinline__ void direct_term_f(float dx, float dy, float dz, float mj, AccF& A, bool comp) {
  const float r2 = dx * dx + dy * dy + dz * dz + 1.0e-20f;
  const float inv = rsqrtf(r2);
  const float inv3 = inv * inv * inv * mj;
  GSPH_ADD_G(A, comp, dx * inv3, dy * inv3, dz * inv3, mj * inv);
}

__device__ __forceinline__ void cell_term_f(const MixedCells& mc, int cc, const TargetF& T, bool quad, AccF& A) {
  const float4 ch = mc.com_hi[cc], cl = mc.com_lo[cc];
  const float dx = (T.ph.x - ch.x) + (T.pl.x - cl.x);
  const float dy = (T.ph.y - ch.y) + (T.pl.y - cl.y);
  const float dz = (T.ph.z - ch.z) + (T.pl.z - cl.z);
  const float r2 = dx * dx + dy * dy + dz * dz + 1.0e-20f;
  const float inv = rsqrtf(r2);
  const float inv2 = inv * inv;
  const float mon = ch.w * inv2 * inv;
  A.ag[0] -= mon * dx; A.ag[1] -= mon * dy; A.ag[2] -= mon * dz;
  A.gpot += ch.w * inv;
  if (quad) {
    const float4 q = mc.quad[cc];
    const float q4 = cl.w;
    const float inv5 = inv2 * inv2 * inv;
    const float qzz = -(q.x + q.z);
    const float qx = q.x * dx + q.y * dy + q.w * dz;
    const float qy = q.y * dx + q.z * dy + q4 * dz;
    const float qz = q.w * dx + q4 * dy + qzz * dz;
    const float qscalar = qx * dx + qy * dy + qz * dz;
    const float qfactor = 2.5f * qscalar * inv5 * inv2;
    A.ag[0] += qx * inv5 - qfactor * dx;
    A.ag[1] += qy * inv5 - qfactor * dy;
    A.ag[2] += qz * inv5 - qfactor * dz;
    A.gpot += 0.5f * qscalar * inv5;
  }
}

// Gravity-walk decision (Tree::ComputeGravityInteractionAndGhostList) for one cell:
// float test with margins, exact fp64 re-test when a float value is inside the margin.
struct LeafGeo {
  float4 hi, lo;                // rcell hi/lo, rmax, hmax
  int c;                        // the leaf cell (its fp64 geometry is read by the exact re-test)
};

template <class Count>
__device__ __forceinline__ int grav_decide(const Tree& t, const MixedCells& mc, const LeafGeo& G, int node, int level,
                                           float4 mt, Count& exact) {
  const int on = __float_as_int(mt.y);
  const float4 gh = mc.geo_hi[node], gl = mc.geo_lo[node];
  const float dx = (gh.x - G.hi.x) + (gl.x - G.lo.x);
  const float dy = (gh.y - G.hi.y) + (gl.y - G.lo.y);
  const float dz = (gh.z - G.hi.z) + (gl.z - G.lo.z);
  const float d2 = dx * dx + dy * dy + dz * dz;
  const float a1 = gh.w + G.hi.w + 2.0f * G.lo.w;
  const float a2 = G.hi.w + gh.w + 2.0f * gl.w;
  const float thr = fmaxf(a1 * a1, a2 * a2);
  int near;
  if (d2 < thr * (1.0f - kMargin)) near = 1;
  else if (d2 > thr * (1.0f + kMargin)) near = 0;
  else near = -1;
  const float cd = mt.x;
  int open_mac;   // 1: too close (open), 0: accept
  if (d2 < cd * (1.0f - kMargin)) open_mac = 1;
  else if (d2 > cd * (1.0f + kMargin)) open_mac = 0;
  else open_mac = -1;
  if (near < 0 || (near == 0 && open_mac < 0)) {
    exact++;
    const CellGeom o = t.geom[node], lg = t.geom[G.c];
    const double ddx = __dsub_rn(o.rcell[0], lg.rcell[0]);
    const double ddy = __dsub_rn(o.rcell[1], lg.rcell[1]);
    const double ddz = __dsub_rn(o.rcell[2], lg.rcell[2]);
    const double drsqd = dot3_rn(ddx, ddy, ddz);
    const double t1 = sq_rn(__dadd_rn(__dadd_rn(o.rmax, lg.rmax), __dmul_rn(kKernRange, lg.hmax)));
    const double t2 = sq_rn(__dadd_rn(__dadd_rn(lg.rmax, o.rmax), __dmul_rn(kKernRange, o.hmax)));
    near = (drsqd <= t1 || drsqd <= t2) ? 1 : 0;
    open_mac = drsqd < o.cdistsqd ? 1 : 0;
  }
  if (near) {
    if (level < t.ltot) return kOpen;
    return on == 0 ? kSkip : kEmitA;
  }
  if (on == 0) return kSkip;
  if (!open_mac) return (level == t.ltot && on == 1) ? kEmitB : kEmitC;
  return level < t.ltot ? kOpen : kEmitB;
}

__device__ __forceinline__ void load_leaf_geo(const Tree& t, const MixedCells& mc, int c, LeafGeo& G) {
  (void) t;
  G.hi = mc.geo_hi[c];
  G.lo = mc.geo_lo[c];
  G.c = c;
}

// lpg: lanes per particle (a power of two, uniform over the warp); the particle's lanes
// are consecutive and the one with sl == 0 writes.
__device__ __forceinline__ void finish_particle_f(const SphParams& prm, const Particles& p, const DeviceCounters& cnt,
                                                  int lpg, bool mine, int sl, int slot, const AccF& A, double gpot0,
                                                  unsigned long long ndir, unsigned long long dhash, bool grav) {
  // the lanes' partial sums added in float (each holds a few hundred float terms already),
  // the per-particle arithmetic after them in float too; results stored as fp64
  float ah[3], ag[3], gp, du, dv;
  double agd[3], gpd;
  for (int k = 0; k < 3; k++) ah[k] = gsum_f(A.ah[k], lpg);
  if (prm.compensated) {   // the lanes' compensated partials combined in fp64
    for (int k = 0; k < 3; k++) agd[k] = gsum_d((double) A.ag[k] - (double) A.cg[k], lpg);
    gpd = gsum_d((double) A.gpot - (double) A.cg[3], lpg);
  } else {
    for (int k = 0; k < 3; k++) { ag[k] = gsum_f(A.ag[k], lpg); agd[k] = ag[k]; }
    gp = gsum_f(A.gpot, lpg);
    gpd = gp;
  }
  du = gsum_f(A.dudt, lpg);
  dv = gsum_f(A.divv, lpg);
  if (cnt.record) {
    unsigned long long dc = ndir, dh = dhash;
    for (int o = 1; o < lpg; o <<= 1) { dc += __shfl_xor_sync(kFull, dc, o); dh += __shfl_xor_sync(kFull, dh, o); }
    if (mine && sl == 0) { atomicAdd(&cnt.rec_dir_cnt[slot], dc); atomicAdd(&cnt.rec_dir_hash[slot], dh); }
  }
  if (!(mine && sl == 0)) return;
  const float rho = (float) p.rho[slot];
  const float invrho = __frcp_rn(rho);
  const float divv = dv * invrho;
  const float P = prm.gm1_f * rho * (float) p.u[slot];
  p.div_v[slot] = (double) divv;
  p.dudt[slot] = (double) (du - P * divv * invrho * (float) p.invomega[slot]);
  p.ax[slot] = (double) ah[0] + agd[0];
  p.ay[slot] = (double) ah[1] + agd[1];
  p.az[slot] = (double) ah[2] + agd[2];
  p.agx[slot] = agd[0]; p.agy[slot] = agd[1]; p.agz[slot] = agd[2];
  p.gpot[slot] = grav ? gpot0 + gpd : 0.0;
}

constexpr int kForceWarps = 4;    // warps per block of the warp-per-leaf force kernels
constexpr int kFStack = 1024;
constexpr int kFListA = 256, kFListB = 128, kFListC = 512;         // warp-per-leaf
constexpr int kWListA = 256, kWListB = 512, kWListC = 1024;         // wide kernel, per warp

// One leaf (or one particle of a leaf) through the gravity walk and all its terms.
// LPG = lanes per particle; pfirst = first particle of the leaf this warp owns.
// give_up: hand the leaf over when the near or direct list overflows.
// Block-shared partial sums of the sliced wide kernel: [slice][particle][9 values].
struct ForceSmem {
  double acc[8][32][9];
  unsigned long long dcnt[8][32], dhash[8][32], ccnt[8], chash[8];
};

// SLICES > 1: the block's SLICES warps share the leaf, each keeping every SLICES-th
// emitted list entry (sel = its slice), and their partial sums are added in slice order.
// REC: the list-recording build (counts, hashes and full lists of every pair kind); the
// production build has none of that code in its pair loops.
// SLICES == 1 hands the leaf over (returns false) when its near or direct list overflows.
template <int LPG, int SLICES, bool REC>
__device__ __forceinline__ bool all_forces_leaf(const Tree& t, const Particles& p, const MixedParticles& mp,
                                                const MixedCells& mc, const SphParams& prm, const DeviceCounters& cnt,
                                                int leaf, int pfirst, int* stack, int* la, int* lb, int* lc, int capa,
                                                int capb, int capc, int sel = 0,
                                                ForceSmem* fs = nullptr) {
  constexpr bool give_up = SLICES == 1;
  const int lane = threadIdx.x & 31;
  constexpr int GT = 32 / LPG;   // particles of the leaf (from pfirst) this warp holds
  const int c = t.leaf_cell[leaf];
  const int first = t.cell_first[c], ncell = t.cell_n[c];
  const bool rec = REC && cnt.record;
  // Lanes to targets.  SLICES == 1: the warp works for the leaf's active particles only,
  // nact of them getting 32 / P consecutive lanes each (P the power of two at or above
  // nact), so that under block timesteps no lane waits on an inactive particle; with every
  // particle active this is LPG lanes per particle in leaf order.  SLICES > 1: LPG lanes
  // per particle of the leaf, active or not (the slices' sums are combined per particle).
  int lpg = LPG, g = lane / LPG, ntg = GT, tk = g;
  bool mine;
  if (SLICES == 1) {
    const unsigned amask =
        __ballot_sync(kFull, lane < GT && pfirst + lane < ncell && is_active(p, first + pfirst + lane));
    if (amask == 0u) return true;   // no active particle in this leaf
    ntg = __popc(amask);
    int pw = 1;
    while (pw < ntg) pw <<= 1;
    lpg = 32 / pw;
    g = lane / lpg;
    mine = g < ntg;
    tk = mine ? nth_bit(amask, g) : 0;
  } else {
    mine = pfirst + g < ncell && is_active(p, first + pfirst + g);
  }
  const int sl = lane % lpg;
  const int pidx = pfirst + tk;
  const int slot = first + (pidx < ncell ? pidx : 0);
  int lvn_own = 0;
  TargetF T;
  load_target_f(p, mp, slot, T);
  LeafGeo G;
  load_leaf_geo(t, mc, c, G);
  const bool quad = prm.multipole == 1;
  AccF A = {};
  // per-lane counts of one leaf fit 32 bits; the hashes and cell counts exist only in the
  // list-recording build
  unsigned nsph = 0, ndir = 0, ndir_b = 0, ncellp = 0, exact = 0;
  unsigned long long dhash = 0, chash = 0, ccount = 0;
  bool gave_up = false;
  // lists have separate capacities: WarpLists keeps one, so the flush test is done here
  WarpLists L{la, lb, lc, 0, 0, 0, 1 << 30};
  // Lists B (direct leaves) and C (multipole cells) run one source per lane against every
  // target particle of the warp: positions relative to the leaf centre (hi + lo pairs,
  // accurate to a few ulps of the separation), 8 targets per round held in registers, the
  // per-target sums reduced over the warp afterwards and added to the target's first lane.
  const float4 lc_hi = mc.geo_hi[c], lc_lo = mc.geo_lo[c];
  auto rel = [&](float4 h, float4 l, float& x, float& y, float& z) {
    x = (h.x - lc_hi.x) + (l.x - lc_lo.x);
    y = (h.y - lc_hi.y) + (l.y - lc_lo.y);
    z = (h.z - lc_hi.z) + (l.z - lc_lo.z);
  };
  // the warp's targets, broadcast from shared memory: leaf-relative position and, in w,
  // 1 + the particle's index in the leaf when active, 0 when not; ntg entries (SLICES == 1:
  // the active particles only, in leaf order)
  constexpr int kTW = SLICES == 1 ? kForceWarps : 8;   // warps per block
  __shared__ float4 s_tgt[kTW][GT];
  float4* tgt = s_tgt[(threadIdx.x >> 5) % kTW];
  {
    float x, y, z;
    rel(T.ph, T.pl, x, y, z);
    if (sl == 0 && g < ntg) tgt[g] = make_float4(x, y, z, mine ? (float) (1 + tk) : 0.0f);
    __syncwarp();
  }
  auto add_to_targets = [&](float (&acc)[8][4], int u0) {
#pragma unroll
    for (int u = 0; u < 8; u++) {
      if (u0 + u >= ntg) break;
      if (SLICES > 1 && tgt[u0 + u].w == 0.0f) continue;   // inactive target: nothing was summed (warp-uniform)
#pragma unroll
      for (int k = 0; k < 4; k++)
        for (int o = 16; o > 0; o >>= 1) acc[u][k] = __fadd_rn(acc[u][k], __shfl_xor_sync(kFull, acc[u][k], o));
      if (lane == (u0 + u) * lpg) {
        if (prm.compensated) {
          kahan_add(A.ag[0], A.cg[0], acc[u][0]); kahan_add(A.ag[1], A.cg[1], acc[u][1]);
          kahan_add(A.ag[2], A.cg[2], acc[u][2]); kahan_add(A.gpot, A.cg[3], acc[u][3]);
        } else {
          A.ag[0] = __fadd_rn(A.ag[0], acc[u][0]); A.ag[1] = __fadd_rn(A.ag[1], acc[u][1]);
          A.ag[2] = __fadd_rn(A.ag[2], acc[u][2]); A.gpot = __fadd_rn(A.gpot, acc[u][3]);
        }
      }
    }
  };
  // targets of the round u0..u0+7 that take terms (the pair counts are kept per source)
  auto round_targets = [&](int u0) {
    unsigned nu = 0;
    for (int u = 0; u < 8 && u0 + u < ntg; u++) nu += (SLICES == 1 || tgt[u0 + u].w != 0.0f) ? 1u : 0u;
    return nu;
  };
  auto consume_c = [&]() {
#pragma unroll
    for (int u0 = 0; u0 < GT; u0 += 8) {
      if (u0 >= ntg) break;
      float acc[8][4] = {};
      const unsigned nu = round_targets(u0);
      for (int e = lane; e < L.nc; e += 32) {
        const int cc = L.c[e];
        const float4 ch = mc.com_hi[cc], cl = mc.com_lo[cc];
        float cx, cy, cz;
        rel(ch, cl, cx, cy, cz);
        const float4 q = quad ? mc.quad[cc] : make_float4(0.f, 0.f, 0.f, 0.f);
        const float q4 = cl.w, qzz = -__fadd_rn(q.x, q.z);
        const float mc_ = ch.w;
#pragma unroll
        for (int u = 0; u < 8; u++) {
          if (u0 + u >= ntg) break;
          const float4 tu = tgt[u0 + u];
          if (SLICES > 1 && tu.w == 0.0f) continue;   // (SLICES == 1: the targets are the active particles)
          // Monopole and quadrupole of the cell (NeighbourSearch.h:423-449) in the form
          //   a += (-m r^-3 - 2.5 (d.Q.d) r^-7) d + r^-5 Q.d,   gpot += m r^-1 + 0.5 (d.Q.d) r^-5,
          // accumulated by fused multiply-adds; explicit roundings: the same sums in every
          // kernel this leaf code is built into
          const float dx = __fsub_rn(tu.x, cx), dy = __fsub_rn(tu.y, cy), dz = __fsub_rn(tu.z, cz);
          const float r2 = __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmaf_rn(dx, dx, 1.0e-20f)));
          const float inv = rsqrtf(r2);
          const float inv2 = __fmul_rn(inv, inv);
          const float minv3 = __fmul_rn(__fmul_rn(mc_, inv), inv2);
          float c1 = -minv3;
          if (quad) {
            const float inv5 = __fmul_rn(__fmul_rn(inv2, inv2), inv);
            const float qx = __fmaf_rn(q.w, dz, __fmaf_rn(q.y, dy, __fmul_rn(q.x, dx)));
            const float qy = __fmaf_rn(q4, dz, __fmaf_rn(q.z, dy, __fmul_rn(q.y, dx)));
            const float qz = __fmaf_rn(qzz, dz, __fmaf_rn(q4, dy, __fmul_rn(q.w, dx)));
            const float qs5 = __fmul_rn(__fmaf_rn(qz, dz, __fmaf_rn(qy, dy, __fmul_rn(qx, dx))), inv5);
            c1 = -__fmaf_rn(__fmul_rn(2.5f, qs5), inv2, minv3);
            acc[u][0] = __fmaf_rn(inv5, qx, acc[u][0]);
            acc[u][1] = __fmaf_rn(inv5, qy, acc[u][1]);
            acc[u][2] = __fmaf_rn(inv5, qz, acc[u][2]);
            acc[u][3] = __fmaf_rn(0.5f, qs5, acc[u][3]);
          }
          acc[u][0] = __fmaf_rn(c1, dx, acc[u][0]);
          acc[u][1] = __fmaf_rn(c1, dy, acc[u][1]);
          acc[u][2] = __fmaf_rn(c1, dz, acc[u][2]);
          acc[u][3] = __fmaf_rn(mc_, inv, acc[u][3]);
        }
        ncellp += nu;
        if (u0 == 0 && rec) {
          chash += mix64((unsigned long long) cc);
          ccount++;
          rec_cell_id(cnt, leaf, cc);
        }
      }
      add_to_targets(acc, u0);
    }
  };
  auto consume_b = [&]() {
#pragma unroll
    for (int u0 = 0; u0 < GT; u0 += 8) {
      if (u0 >= ntg) break;
      float acc[8][4] = {};
      const unsigned nu = round_targets(u0);
      for (int e0 = 0; e0 < L.nb; e0 += LPG) {
        const int e = e0 + lane / GT, q = lane % GT;
        if (e >= L.nb) continue;
        const unsigned lw = (unsigned) L.b[e];
        if (q >= leaf_count(lw)) continue;
        const int j = leaf_first(lw) + q;
        const float4 pjh = mp.pos_hi[j], pjl = mp.pos_lo[j];
        float sx, sy, sz;
        rel(pjh, pjl, sx, sy, sz);
        const float mj = pjh.w;
        ndir_b += nu;
#pragma unroll
        for (int u = 0; u < 8; u++) {
          if (u0 + u >= ntg) break;
          const float4 tu = tgt[u0 + u];
          if (SLICES > 1 && tu.w == 0.0f) continue;
          const float dx = __fsub_rn(sx, tu.x), dy = __fsub_rn(sy, tu.y), dz = __fsub_rn(sz, tu.z);
          const float r2 = __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmaf_rn(dx, dx, 1.0e-20f)));
          const float inv = rsqrtf(r2);
          const float minv = __fmul_rn(mj, inv);
          const float inv3 = __fmul_rn(__fmul_rn(inv, inv), minv);
          acc[u][0] = __fmaf_rn(dx, inv3, acc[u][0]); acc[u][1] = __fmaf_rn(dy, inv3, acc[u][1]);
          acc[u][2] = __fmaf_rn(dz, inv3, acc[u][2]); acc[u][3] = __fadd_rn(acc[u][3], minv);
          if (rec) {
            const int ts = first + pfirst + (int) tu.w - 1;
            atomicAdd(&cnt.rec_dir_cnt[ts], 1ull);
            atomicAdd(&cnt.rec_dir_hash[ts], mix64((unsigned long long) p.id[j]));
            rec_direct_id(cnt, ts, p.id[j]);
          }
        }
      }
      add_to_targets(acc, u0);
    }
  };
  // near leaves: the particle's lpg lanes take the (entry, particle) pairs of the list in
  // turn (for lpg <= GT, particle q of every entry goes to lane q mod lpg)
  auto near_pair = [&](int j) {
    const float4 pjh = mp.pos_hi[j], pjl = mp.pos_lo[j];
    const float dx = (pjh.x - T.ph.x) + (pjl.x - T.pl.x);
    const float dy = (pjh.y - T.ph.y) + (pjl.y - T.pl.y);
    const float dz = (pjh.z - T.ph.z) + (pjl.z - T.pl.z);
    const float d2 = dx * dx + dy * dy + dz * dz;
    const float4 vj = mp.vel[j], hj = mp.hyd[j], xj = mp.aux[j];
    if (sph_member(p, T, j, d2, pjl.w, prm, exact)) {
      hydro_grav_pair_f(prm, T, vj, hj, xj, dx, dy, dz, d2, pjh.w, A);
      lvn_pair(p, slot, j, lvn_own);
      nsph++;
      if (rec) {
        const int k = atomicAdd(&cnt.rec_sph_cnt[slot], 1);
        if (k < cnt.rec_max) cnt.rec_sph_ids[(size_t) slot * cnt.rec_max + k] = j;
      }
    } else {
      direct_term_f(dx, dy, dz, pjh.w, A, prm.compensated != 0);
      ndir++;
      if (rec) {
        dhash += mix64((unsigned long long) p.id[j]);
        rec_direct_id(cnt, slot, p.id[j]);
      }
    }
  };
  auto consume_ab = [&]() {
    if (!mine) return;
    const int ntot = L.na * GT;
    for (int idx = sl; idx < ntot; idx += lpg) {
      const unsigned lw = (unsigned) L.a[idx / GT];
      const int qq = idx % GT;
      if (qq < leaf_count(lw)) near_pair(leaf_first(lw) + qq);
    }
  };
  // the walk, with per-list flushing
  const unsigned lt = (1u << lane) - 1u;
  if (lane == 0) stack[0] = 0;
  int top = 1;
  bool stack_ok = true;
  int ea = 0, eb = 0, ec = 0;   // entries emitted so far (slicing)
  __syncwarp();
  while (top > 0) {
    const int take = top < 32 ? top : 32;
    int node = -1;
    if (lane < take) node = stack[top - 1 - lane];
    top -= take;
    __syncwarp();
    int act = kSkip, level = 0;
    unsigned lw = 0;   // the leaf's list word (near and direct-sum entries)
    if (node >= 0) {
      const float4 mt = mc.meta[node];
      level = __float_as_int(mt.z);
      act = grav_decide(t, mc, G, node, level, mt, exact);
      lw = pack_leaf(__float_as_int(mt.w), __float_as_int(mt.y));
    }
    const unsigned mo = __ballot_sync(kFull, act == kOpen);
    const int nopen = __popc(mo);
    if (top + 2 * nopen > kFStack) { stack_ok = false; break; }
    if (act == kOpen) {
      const int r = __popc(mo & lt);
      stack[top + 2 * r] = c2_of(node, level, t.ltot);
      stack[top + 2 * r + 1] = node + 1;
    }
    top += 2 * nopen;
    bool ka = act == kEmitA, kb = act == kEmitB, kc = act == kEmitC;
    if (SLICES > 1) {
      const unsigned xa = __ballot_sync(kFull, ka), xb = __ballot_sync(kFull, kb), xc = __ballot_sync(kFull, kc);
      ka = ka && ((ea + __popc(xa & lt)) % SLICES == sel);
      kb = kb && ((eb + __popc(xb & lt)) % SLICES == sel);
      kc = kc && ((ec + __popc(xc & lt)) % SLICES == sel);
      ea += __popc(xa); eb += __popc(xb); ec += __popc(xc);
    }
    const unsigned ma = __ballot_sync(kFull, ka);
    const unsigned mb = __ballot_sync(kFull, kb);
    const unsigned mcm = __ballot_sync(kFull, kc);
    if (ka) L.a[L.na + __popc(ma & lt)] = (int) lw;
    if (kb) L.b[L.nb + __popc(mb & lt)] = (int) lw;
    if (kc) L.c[L.nc + __popc(mcm & lt)] = node;
    L.na += __popc(ma); L.nb += __popc(mb); L.nc += __popc(mcm);
    __syncwarp();
    if (L.nc > capc - 32) { consume_c(); L.nc = 0; __syncwarp(); }
    if (L.na > capa - 32 || L.nb > capb - 32) {
      if constexpr (give_up) {
        gave_up = true;
        break;
      } else {
        consume_ab(); consume_b(); L.na = 0; L.nb = 0; __syncwarp();
      }
    }
  }
  if (gave_up) {
    // cells already consumed are recorded again by the kernel that takes the leaf over
    if (rec && cnt.rec_cell_ids && lane == 0) cnt.rec_cell_n[leaf] = 0;
    return false;
  }
  consume_ab();
  consume_b();
  consume_c();
  lvn_finish(p, slot, mine, lvn_own);
  if (!stack_ok && lane == 0) atomicOr(cnt.status, (unsigned) kStatusStackOverflow);
  unsigned long long a1 = nsph, a2 = ndir + ndir_b, a3 = ncellp, a4 = exact;
  for (int o = 16; o > 0; o >>= 1) {
    a1 += __shfl_xor_sync(kFull, a1, o); a2 += __shfl_xor_sync(kFull, a2, o);
    a3 += __shfl_xor_sync(kFull, a3, o); a4 += __shfl_xor_sync(kFull, a4, o);
  }
  if (lane == 0) {
    atomicAdd(cnt.hydro_pairs, a1); atomicAdd(cnt.direct_pairs, a2);
    atomicAdd(cnt.cell_pairs, a3); atomicAdd(cnt.exact_checks, a4);
  }
  unsigned long long cc = ccount, ch = chash;
  if (rec) {
    for (int o = 16; o > 0; o >>= 1) { cc += __shfl_xor_sync(kFull, cc, o); ch += __shfl_xor_sync(kFull, ch, o); }
  }
  const double gpot0 = (double) (T.ph.w * T.hyd.x * (float) m4_wpot(0.0));   // (m / h) wpot(0)
  if (SLICES == 1) {
    if (rec && pfirst == 0 && lane == 0) { cnt.rec_cell_cnt[leaf] = cc; cnt.rec_cell_hash[leaf] = ch; }
    finish_particle_f(prm, p, cnt, lpg, mine, sl, slot, A, gpot0, ndir, dhash, true);
    return true;
  }
  // sliced: reduce each particle inside the warp, then across slices in slice order
  double v[9];
  // (the compensation terms are zero unless the sums are compensated)
  for (int k = 0; k < 3; k++) { v[k] = (double) A.ah[k]; v[3 + k] = (double) A.ag[k] - (double) A.cg[k]; }
  v[6] = (double) A.gpot - (double) A.cg[3]; v[7] = A.dudt; v[8] = A.divv;
  unsigned long long dc = ndir, dh = dhash;
  for (int o = 1; o < LPG; o <<= 1) {
    for (int k = 0; k < 9; k++) v[k] += __shfl_xor_sync(kFull, v[k], o);
    dc += __shfl_xor_sync(kFull, dc, o);
    dh += __shfl_xor_sync(kFull, dh, o);
  }
  if (sl == 0) {
    for (int k = 0; k < 9; k++) fs->acc[sel][g][k] = v[k];
    fs->dcnt[sel][g] = dc;
    fs->dhash[sel][g] = dh;
  }
  if (lane == 0) { fs->ccnt[sel] = cc; fs->chash[sel] = ch; }
  __syncthreads();
  if (sel == 0) {
    if (mine && sl == 0) {
      double tot[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
      unsigned long long tdc = 0, tdh = 0;
      for (int w = 0; w < SLICES; w++) {
        for (int k = 0; k < 9; k++) tot[k] += fs->acc[w][g][k];
        tdc += fs->dcnt[w][g];
        tdh += fs->dhash[w][g];
      }
      if (rec) { atomicAdd(&cnt.rec_dir_cnt[slot], tdc); atomicAdd(&cnt.rec_dir_hash[slot], tdh); }
      const double rho = p.rho[slot];
      const double invrho = 1.0 / rho;
      const double divv = tot[8] * invrho;
      const double P = (prm.gamma_eos - 1.0) * rho * p.u[slot];
      p.div_v[slot] = divv;
      p.dudt[slot] = tot[7] - P * divv * invrho * p.invomega[slot];
      p.ax[slot] = tot[0] + tot[3]; p.ay[slot] = tot[1] + tot[4]; p.az[slot] = tot[2] + tot[5];
      p.agx[slot] = tot[3]; p.agy[slot] = tot[4]; p.agz[slot] = tot[5];
      p.gpot[slot] = gpot0 + tot[6];
    }
    if (rec && lane == 0) {
      unsigned long long tc = 0, th = 0;
      for (int w = 0; w < SLICES; w++) { tc += fs->ccnt[w]; th += fs->chash[w]; }
      cnt.rec_cell_cnt[leaf] = tc;
      cnt.rec_cell_hash[leaf] = th;
    }
  }
  __syncthreads();
  return true;
}

// Five blocks (20 warps) per SM: the walk and the list loads are latency bound, and at four
// blocks an SM (128 registers) the 1M rotating-cloud force pass took 10 % longer.  The
// target's and the leaf's fp64 copies are read only where the exact re-tests need them, so
// the kernel fits 94 registers (16 bytes of spill).
template <int LPG, bool REC>
__global__ void __launch_bounds__(kForceWarps * 32, 5)
k_all_forces_mixed(Tree t, Particles p, MixedParticles mp, MixedCells mc, SphParams prm, DeviceCounters cnt,
                   HeavyList heavy) {
  __shared__ int s_stack[kForceWarps][kFStack];
  __shared__ int s_a[kForceWarps][kFListA];
  __shared__ int s_b[kForceWarps][kFListB];
  __shared__ int s_c[kForceWarps][kFListC];
  const int wib = threadIdx.x >> 5;
  const int leaf = blockIdx.x * kForceWarps + wib;
  if (leaf >= t.nleaf) return;
  const bool ok = all_forces_leaf<LPG, 1, REC>(t, p, mp, mc, prm, cnt, leaf, 0, s_stack[wib], s_a[wib], s_b[wib],
                                               s_c[wib], tuned_depth(prm.near_depth, 64, kFListA), kFListB,
                                               tuned_depth(prm.cell_depth, 64, kFListC));
  if (!ok && (threadIdx.x & 31) == 0) {
    const int k = atomicAdd(heavy.count, 1);
    heavy.leaves[k] = leaf;
  }
}

// Heavy leaves: the block's 8 warps share each leaf, each taking an eighth of its
// near-leaf, direct-leaf and cell lists for all of its particles.
template <int LPG, bool REC>
__global__ void __launch_bounds__(256)
k_all_forces_mixed_wide(Tree t, Particles p, MixedParticles mp, MixedCells mc, SphParams prm, DeviceCounters cnt,
                        HeavyList heavy) {
  extern __shared__ int s_dyn[];
  const int wib = threadIdx.x >> 5;
  const int per = kFStack + kWListA + kWListB + kWListC;
  int* base = s_dyn + wib * per;
  ForceSmem* fs = reinterpret_cast<ForceSmem*>(s_dyn + 8 * per);
  const int nh = *heavy.count;
  for (int k = blockIdx.x; k < nh; k += gridDim.x) {
    all_forces_leaf<LPG, 8, REC>(t, p, mp, mc, prm, cnt, heavy.leaves[k], 0, base, base + kFStack, base + kFStack + kWListA,
                            base + kFStack + kWListA + kWListB, kWListA, kWListB, kWListC, wib, fs);
  }
}

// ---- hydro only (periodic or open), warp per leaf ----------------------------------------
constexpr int kHListA = 512;

template <int LPG>
__device__ __forceinline__ void hydro_leaf(const Tree& t, const Particles& p, const MixedParticles& mp,
                                           const MixedCells& mc, const SphParams& prm, const DeviceCounters& cnt,
                                           int leaf, int* stack, int* list) {
  const int lane = threadIdx.x & 31;
  const int g = lane / LPG, sl = lane % LPG;
  const int c = t.leaf_cell[leaf];
  const int first = t.cell_first[c], ncell = t.cell_n[c];
  const bool mine = g < ncell && is_active(p, first + g);
  if (!__any_sync(kFull, mine)) return;   // no active particle in this leaf
  const int slot = first + (g < ncell ? g : 0);
  TargetF T;
  load_target_f(p, mp, slot, T);
  AccF A = {};
  unsigned long long npairs = 0, exact = 0;
  int lvn_own = 0;
  WarpLists L{list, list, list, 0, 0, 0, kHListA};
  const float4 bmin_f = mc.bbmin[c], bmax_f = mc.bbmax[c], hmin_f = mc.hbmin[c], hmax_f = mc.hbmax[c];
  const float half[3] = {(float) prm.boxhalf[0], (float) prm.boxhalf[1], (float) prm.boxhalf[2]};
  const float size[3] = {(float) prm.boxsize[0], (float) prm.boxsize[1], (float) prm.boxsize[2]};
  // Superset of the reference's PeriodicBoxOverlap: along each axis the boxes overlap
  // for some periodic image of the second (outward-rounded float boxes, widened by a
  // margin of the box size); membership is decided per pair afterwards.
  auto pbox = [&](float4 amin, float4 amax, float4 bmin, float4 bmax) -> bool {
    const float a0[3] = {amin.x, amin.y, amin.z}, a1[3] = {amax.x, amax.y, amax.z};
    const float b0[3] = {bmin.x, bmin.y, bmin.z}, b1[3] = {bmax.x, bmax.y, bmax.z};
    for (int k = 0; k < 3; k++) {
      bool ok = !(a0[k] > b1[k] || b0[k] > a1[k]);
      if (!ok && prm.periodic) {
        const float slack = size[k] * kMargin;
        for (int sgn = -1; sgn <= 1 && !ok; sgn += 2) {
          const float lo = b0[k] + sgn * size[k] - slack, hi = b1[k] + sgn * size[k] + slack;
          ok = !(a0[k] > hi || lo > a1[k]);
        }
      }
      if (!ok) return false;
    }
    return true;
  };
  auto decide = [&](int node, int& level) -> int {
    const float4 b0 = mc.bbmin[node], b1 = mc.bbmax[node];   // w: cell_n, first << 5 | level
    level = box_level(b1.w);
    if (__float_as_int(b0.w) == 0) return kSkip;
    if (!(pbox(bmin_f, bmax_f, mc.hbmin[node], mc.hbmax[node]) || pbox(hmin_f, hmax_f, b0, b1)))
      return kSkip;
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
        const float4 pjh = mp.pos_hi[j], pjl = mp.pos_lo[j];
        float d[3] = {(pjh.x - T.ph.x) + (pjl.x - T.pl.x), (pjh.y - T.ph.y) + (pjl.y - T.pl.y),
                      (pjh.z - T.ph.z) + (pjl.z - T.pl.z)};
        if (prm.periodic) {
          const double xj[3] = {p.x[j], p.y[j], p.z[j]}, xi[3] = {p.x[slot], p.y[slot], p.z[slot]};
          int sh[3] = {0, 0, 0};   // image of j, in box lengths
          for (int k = 0; k < 3; k++) {
            if (fabsf(d[k]) > half[k] * 0.5f) {
              double dd = xj[k] - xi[k];
              if (dd > prm.boxhalf[k]) { dd -= prm.boxsize[k]; sh[k] = -1; }
              else if (dd < -prm.boxhalf[k]) { dd += prm.boxsize[k]; sh[k] = 1; }
              d[k] = (float) dd;
            }
          }
          if ((sh[0] | sh[1] | sh[2]) && !ghost_exists(prm, p, j, sh)) continue;
        }
        const float d2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
        if (!sph_member(p, T, j, d2, pjl.w, prm, exact)) continue;
        hydro_pair_f(prm, mp, T, j, d[0], d[1], d[2], d2, pjh.w, A);
        lvn_pair(p, slot, j, lvn_own);
        npairs++;
        if (cnt.record) {
          const int k = atomicAdd(&cnt.rec_sph_cnt[slot], 1);
          if (k < cnt.rec_max) cnt.rec_sph_ids[(size_t) slot * cnt.rec_max + k] = j;
        }
      }
    }
  };
  const bool ok = warp_walk_lv(0, t.ltot, stack, kFStack, L, decide, tag, consume);
  consume();
  if (!ok && lane == 0) atomicOr(cnt.status, (unsigned) kStatusStackOverflow);
  unsigned long long a1 = npairs, a4 = exact;
  for (int o = 16; o > 0; o >>= 1) { a1 += __shfl_xor_sync(kFull, a1, o); a4 += __shfl_xor_sync(kFull, a4, o); }
  if (lane == 0) { atomicAdd(cnt.hydro_pairs, a1); atomicAdd(cnt.exact_checks, a4); }
  lvn_finish(p, slot, mine, lvn_own);
  finish_particle_f(prm, p, cnt, LPG, mine, sl, slot, A, 0.0, 0, 0, false);
}

template <int LPG>
__global__ void __launch_bounds__(kForceWarps * 32)
k_hydro_mixed(Tree t, Particles p, MixedParticles mp, MixedCells mc, SphParams prm, DeviceCounters cnt) {
  __shared__ int s_stack[kForceWarps][kFStack];
  __shared__ int s_list[kForceWarps][kHListA];
  const int wib = threadIdx.x >> 5;
  const int leaf = blockIdx.x * kForceWarps + wib;
  if (leaf >= t.nleaf) return;
  hydro_leaf<LPG>(t, p, mp, mc, prm, cnt, leaf, s_stack[wib], s_list[wib]);
}

// ==========================================================================================
// Batched passes over many simulations (batch.cuh).
// ==========================================================================================
// Largest s with start[s] <= item (start has nsim + 1 nondecreasing entries).
__device__ __forceinline__ int find_sim(const int* start, int nsim, int item) {
  int lo = 0, hi = nsim - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (start[mid] <= item) lo = mid; else hi = mid - 1;
  }
  return lo;
}

__device__ __forceinline__ int warp_take(int* counter) {
  int item = 0;
  if ((threadIdx.x & 31) == 0) item = atomicAdd(counter, 1);
  return __shfl_sync(kFull, item, 0);
}

__device__ __forceinline__ int block_take(int* counter, int* s_item) {
  __syncthreads();
  if (threadIdx.x == 0) *s_item = atomicAdd(counter, 1);
  __syncthreads();
  return *s_item;
}

__global__ void k_batch_heavy_prefix(BatchQueue q) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  int acc = 0;
  for (int s = 0; s < q.nsim; s++) {
    q.heavy_start[s] = acc;
    acc += *q.sims[s].heavy.count;
  }
  q.heavy_start[q.nsim] = acc;
}

template <int LPG>
__global__ void __launch_bounds__(kDensWarps * 32, 3) k_batch_density(BatchQueue q) {
  extern __shared__ float2 s_dyn2[];
  float2* s_compact = s_dyn2;
  int* s_stack = reinterpret_cast<int*>(s_dyn2 + kDensWarps * kCompactPerWarp);
  int* s_list = s_stack + kDensWarps * kDensStack;
  const int wib = threadIdx.x >> 5;
  const int kcap = compact_stride(LPG, kCompactPerWarp);
  const int total = q.leaf_start[q.nsim];
  for (;;) {
    const int item = warp_take(&q.next[0]);
    if (item >= total) break;
    const int s = find_sim(q.leaf_start, q.nsim, item);
    const SimDesc& d = q.sims[s];
    const int leaf = item - q.leaf_start[s];
    const bool ok = density_cell<LPG, 1>(d.t, d.p, d.mp, d.mc, d.prm, d.cnt, leaf, s_stack + wib * kDensStack,
                                         s_list + wib * kDensListNormal,
                                         tuned_depth(d.prm.gather_depth, 64, kDensListNormal),
                                         s_compact + wib * kCompactPerWarp, kcap, true, nullptr);
    if (!ok && (threadIdx.x & 31) == 0) {
      const int k = atomicAdd(d.heavy.count, 1);
      d.heavy.leaves[k] = leaf;
    }
  }
}

template <int LPG>
__global__ void __launch_bounds__(256, 2) k_batch_density_pp(BatchQueue q) {
  __shared__ PPShared sm;
  __shared__ int s_item;
  const int total = q.heavy_start[q.nsim];
  for (;;) {
    const int item = block_take(&q.next[1], &s_item);
    if (item >= total) break;
    const int s = find_sim(q.heavy_start, q.nsim, item);
    const SimDesc& d = q.sims[s];
    density_pp_leaf<LPG>(d.t, d.p, d.mp, d.mc, d.prm, d.cnt, d.heavy.leaves[item - q.heavy_start[s]], sm);
  }
}

template <int LPG>
__global__ void __launch_bounds__(kForceWarps * 32) k_batch_hydro(BatchQueue q) {
  __shared__ int s_stack[kForceWarps][kFStack];
  __shared__ int s_list[kForceWarps][kHListA];
  const int wib = threadIdx.x >> 5;
  const int total = q.leaf_start[q.nsim];
  for (;;) {
    const int item = warp_take(&q.next[2]);
    if (item >= total) break;
    const int s = find_sim(q.leaf_start, q.nsim, item);
    const SimDesc& d = q.sims[s];
    hydro_leaf<LPG>(d.t, d.p, d.mp, d.mc, d.prm, d.cnt, item - q.leaf_start[s], s_stack[wib], s_list[wib]);
  }
}

template <int LPG, bool REC>
__global__ void __launch_bounds__(kForceWarps * 32, 5) k_batch_forces(BatchQueue q) {
  __shared__ int s_stack[kForceWarps][kFStack];
  __shared__ int s_a[kForceWarps][kFListA];
  __shared__ int s_b[kForceWarps][kFListB];
  __shared__ int s_c[kForceWarps][kFListC];
  const int wib = threadIdx.x >> 5;
  const int total = q.leaf_start[q.nsim];
  for (;;) {
    const int item = warp_take(&q.next[2]);
    if (item >= total) break;
    const int s = find_sim(q.leaf_start, q.nsim, item);
    const SimDesc& d = q.sims[s];
    const int leaf = item - q.leaf_start[s];
    const bool ok = all_forces_leaf<LPG, 1, REC>(d.t, d.p, d.mp, d.mc, d.prm, d.cnt, leaf, 0, s_stack[wib], s_a[wib],
                                            s_b[wib], s_c[wib], tuned_depth(d.prm.near_depth, 64, kFListA), kFListB,
                                            tuned_depth(d.prm.cell_depth, 64, kFListC));
    if (!ok && (threadIdx.x & 31) == 0) {
      const int k = atomicAdd(d.heavy.count, 1);
      d.heavy.leaves[k] = leaf;
    }
  }
}

template <int LPG, bool REC>
__global__ void __launch_bounds__(256) k_batch_forces_wide(BatchQueue q) {
  extern __shared__ int s_dyn[];
  __shared__ int s_item;
  const int wib = threadIdx.x >> 5;
  const int per = kFStack + kWListA + kWListB + kWListC;
  int* base = s_dyn + wib * per;
  ForceSmem* fs = reinterpret_cast<ForceSmem*>(s_dyn + 8 * per);
  const int total = q.heavy_start[q.nsim];
  for (;;) {
    const int item = block_take(&q.next[3], &s_item);
    if (item >= total) break;
    const int s = find_sim(q.heavy_start, q.nsim, item);
    const SimDesc& d = q.sims[s];
    all_forces_leaf<LPG, 8, REC>(d.t, d.p, d.mp, d.mc, d.prm, d.cnt, d.heavy.leaves[item - q.heavy_start[s]], 0, base,
                            base + kFStack, base + kFStack + kWListA, base + kFStack + kWListA + kWListB, kWListA,
                            kWListB, kWListC, wib, fs);
  }
}

int grid1(int n) { return n < 1 ? 1 : (n + 255) / 256 < 152 * 8 ? (n + 255) / 256 : 152 * 8; }

}  // namespace

int mixed_max_particles() { return kMixedMaxParticles; }

void launch_mixed_prep_build(const Tree& t, const Particles& p, const MixedParticles& mp, const MixedCells& mc,
                             cudaStream_t st) {
  k_prep_build_particles<<<grid1(p.n), 256, 0, st>>>(p, mp);
  k_prep_build_cells<<<grid1(t.ncell), 256, 0, st>>>(t, mc);
}

void launch_mixed_prep_hydro(const Tree& t, const Particles& p, const MixedParticles& mp, const MixedCells& mc,
                             cudaStream_t st) {
  k_prep_hydro_particles<<<grid1(p.n), 256, 0, st>>>(p, mp);
  k_prep_hydro_cells<<<grid1(t.ncell), 256, 0, st>>>(t, mc);
}

#define GSPH_MIXED_LPG(KERNEL, LPG, GRID, BLOCK, SMEM, ...)                               \
  switch (LPG) {                                                                         \
    case 32: KERNEL<32><<<GRID, BLOCK, SMEM, st>>>(__VA_ARGS__); break;                  \
    case 16: KERNEL<16><<<GRID, BLOCK, SMEM, st>>>(__VA_ARGS__); break;                  \
    case 8: KERNEL<8><<<GRID, BLOCK, SMEM, st>>>(__VA_ARGS__); break;                    \
    case 4: KERNEL<4><<<GRID, BLOCK, SMEM, st>>>(__VA_ARGS__); break;                    \
    case 2: KERNEL<2><<<GRID, BLOCK, SMEM, st>>>(__VA_ARGS__); break;                    \
    default: KERNEL<1><<<GRID, BLOCK, SMEM, st>>>(__VA_ARGS__); break;                   \
  }

// Kernels with a recording variant: REC is a compile-time constant at each call.
#define GSPH_MIXED_LPG_REC(KERNEL, REC, LPG, GRID, BLOCK, SMEM, ...)                      \
  switch (LPG) {                                                                         \
    case 32: KERNEL<32, REC><<<GRID, BLOCK, SMEM, st>>>(__VA_ARGS__); break;             \
    case 16: KERNEL<16, REC><<<GRID, BLOCK, SMEM, st>>>(__VA_ARGS__); break;             \
    case 8: KERNEL<8, REC><<<GRID, BLOCK, SMEM, st>>>(__VA_ARGS__); break;               \
    case 4: KERNEL<4, REC><<<GRID, BLOCK, SMEM, st>>>(__VA_ARGS__); break;               \
    case 2: KERNEL<2, REC><<<GRID, BLOCK, SMEM, st>>>(__VA_ARGS__); break;               \
    default: KERNEL<1, REC><<<GRID, BLOCK, SMEM, st>>>(__VA_ARGS__); break;              \
  }

template <bool REC>
void set_wide_smem(bool batch, size_t smem) {
  if (batch) {
    for (auto f : {k_batch_forces_wide<1, REC>, k_batch_forces_wide<2, REC>, k_batch_forces_wide<4, REC>,
                   k_batch_forces_wide<8, REC>, k_batch_forces_wide<16, REC>, k_batch_forces_wide<32, REC>})
      cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem);
  } else {
    for (auto f : {k_all_forces_mixed_wide<1, REC>, k_all_forces_mixed_wide<2, REC>, k_all_forces_mixed_wide<4, REC>,
                   k_all_forces_mixed_wide<8, REC>, k_all_forces_mixed_wide<16, REC>, k_all_forces_mixed_wide<32, REC>})
      cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem);
  }
}

int launch_density_mixed(const Tree& t, const Particles& p, const MixedParticles& mp, const MixedCells& mc,
                         const SphParams& prm, const DeviceCounters& cnt, const HeavyList& heavy,
                         const HeavyList& wide, int lanes_per_particle, int max_leaf, cudaStream_t st) {
  cudaMemsetAsync(heavy.count, 0, sizeof(int), st);
  cudaMemsetAsync(wide.count, 0, sizeof(int), st);
  (void) max_leaf;
  // every leaf, normal lists; overflowing leaves to the wide tier
  GSPH_MIXED_LPG(k_density_mixed, lanes_per_particle, t.nleaf, 32, dens_smem(1, kCompactNormal), t, p, mp, mc, prm,
                 cnt, wide, (const int*) nullptr, (const int*) nullptr, kCompactNormal)
  // the wide tier's leaves, up to 32 one-warp blocks an SM taking the entries in a strided
  // loop (blocks past the count return at once, and the block scheduler balances leaves of
  // uneven cost: 262k Plummer, about 4,900 such leaves, 2.17 -> 2.03 ms with this grid
  // against 13 blocks an SM), overflow to the heavy kernel
  const int wgrid = t.nleaf < 32 * 152 ? t.nleaf : 32 * 152;
  GSPH_MIXED_LPG(k_density_mixed, lanes_per_particle, wgrid, 32, dens_smem(1, kCompactWide), t, p, mp, mc, prm,
                 cnt, heavy, wide.leaves, wide.count, kCompactWide)
  // 41 KB of shared memory a block: up to 5 blocks an SM; 4 per SM keep the heavy leaves
  // (a few percent of all) spread over every SM
  GSPH_MIXED_LPG(k_density_mixed_pp, lanes_per_particle, 4 * 152, 256, 0, t, p, mp, mc, prm, cnt, heavy)
  return 3;
}

int launch_all_forces_mixed(const Tree& t, const Particles& p, const MixedParticles& mp, const MixedCells& mc,
                            const SphParams& prm, const DeviceCounters& cnt, const HeavyList& heavy,
                            int lanes_per_particle, int max_leaf, cudaStream_t st) {
  cudaMemsetAsync(heavy.count, 0, sizeof(int), st);
  const int blocks = (t.nleaf + kForceWarps - 1) / kForceWarps;
  const size_t smem = sizeof(int) * 8 * (kFStack + kWListA + kWListB + kWListC) + sizeof(ForceSmem);
  (void) max_leaf;
  if (cnt.record) {
    GSPH_MIXED_LPG_REC(k_all_forces_mixed, true, lanes_per_particle, blocks, kForceWarps * 32, 0, t, p, mp, mc, prm,
                       cnt, heavy)
    set_wide_smem<true>(false, smem);
    GSPH_MIXED_LPG_REC(k_all_forces_mixed_wide, true, lanes_per_particle, 152 * 2, 256, smem, t, p, mp, mc, prm, cnt,
                       heavy)
  } else {
    GSPH_MIXED_LPG_REC(k_all_forces_mixed, false, lanes_per_particle, blocks, kForceWarps * 32, 0, t, p, mp, mc, prm,
                       cnt, heavy)
    set_wide_smem<false>(false, smem);
    GSPH_MIXED_LPG_REC(k_all_forces_mixed_wide, false, lanes_per_particle, 152 * 2, 256, smem, t, p, mp, mc, prm, cnt,
                       heavy)
  }
  return 2;
}

int launch_hydro_mixed(const Tree& t, const Particles& p, const MixedParticles& mp, const MixedCells& mc,
                       const SphParams& prm, const DeviceCounters& cnt, int lanes_per_particle, cudaStream_t st) {
  const int blocks = (t.nleaf + kForceWarps - 1) / kForceWarps;
  GSPH_MIXED_LPG(k_hydro_mixed, lanes_per_particle, blocks, kForceWarps * 32, 0, t, p, mp, mc, prm, cnt)
  return 1;
}

int launch_batch_density(const BatchQueue& q, int lpg, cudaStream_t st) {
  cudaMemsetAsync(q.next, 0, 4 * sizeof(int), st);
  const size_t smem_n = dens_smem(kDensWarps);
  for (auto f : {k_batch_density<1>, k_batch_density<2>, k_batch_density<4>, k_batch_density<8>,
                 k_batch_density<16>, k_batch_density<32>})
    cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem_n);
  GSPH_MIXED_LPG(k_batch_density, lpg, 152 * 3, kDensWarps * 32, smem_n, q)
  k_batch_heavy_prefix<<<1, 32, 0, st>>>(q);
  GSPH_MIXED_LPG(k_batch_density_pp, lpg, 152 * 2, 256, 0, q)
  return 3;
}

int launch_batch_forces(const BatchQueue& q, bool gravity, int lpg, cudaStream_t st) {
  if (!gravity) {
    GSPH_MIXED_LPG(k_batch_hydro, lpg, 152 * 4, kForceWarps * 32, 0, q)
    return 1;
  }
  const size_t smem = sizeof(int) * 8 * (kFStack + kWListA + kWListB + kWListC) + sizeof(ForceSmem);
  if (q.record) {
    GSPH_MIXED_LPG_REC(k_batch_forces, true, lpg, 152 * 5, kForceWarps * 32, 0, q)
    k_batch_heavy_prefix<<<1, 32, 0, st>>>(q);
    set_wide_smem<true>(true, smem);
    GSPH_MIXED_LPG_REC(k_batch_forces_wide, true, lpg, 152 * 2, 256, smem, q)
  } else {
    GSPH_MIXED_LPG_REC(k_batch_forces, false, lpg, 152 * 5, kForceWarps * 32, 0, q)
    k_batch_heavy_prefix<<<1, 32, 0, st>>>(q);
    set_wide_smem<false>(true, smem);
    GSPH_MIXED_LPG_REC(k_batch_forces_wide, false, lpg, 152 * 2, 256, smem, q)
  }
  return 3;
}


}  // namespace gsph
