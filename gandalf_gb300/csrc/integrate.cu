// Device KDK leapfrog and block timesteps (integrate.cuh).
//
//  k_kdk_begin      SphSimulation::MainLoop time advance      src/Hydrodynamics/SphSimulation.cpp:585-590
//  k_kdk_advance    SphLeapfrogKDK::AdvanceParticles          src/Hydrodynamics/SphLeapfrogKDK.cpp:76-130
//                   + TimeIntegration::CheckBoundaries         src/Common/Integration.cpp:11-80
//  k_kdk_check      unset active + SphLeapfrogKDK::CheckTimesteps  SphLeapfrogKDK.cpp:284-331
//  k_bt_*           Simulation::ComputeBlockTimesteps          src/Common/Simulation.cpp:1764-2190
//                   (Nlevels = 1: ComputeGlobalTimestep        :1666-1752)
//                   with SphIntegration::Timestep              src/Hydrodynamics/SphIntegration.cpp:81-130
//  k_kdk_end        SphLeapfrogKDK::EndTimestep                SphLeapfrogKDK.cpp:219-275
// The arithmetic of every update is written unfused, in the reference's operand order.
#include "integrate.cuh"

namespace gsph {
namespace {

constexpr double kSmallDp = 1.0e-50;          // small_number_dp, src/Headers/Constants.h:90
constexpr double kInvLogTwo = 1.44269504088896;  // invlogetwo, src/Headers/Constants.h:64

__device__ __forceinline__ int pow2i(int k) { return k >= 0 ? (1 << k) : 0; }   // (int) pow(2, k)

// ComputeTimestepLevel (src/Headers/InlineFuncs.h:550-557): (int) (invlogetwo log q) + 1,
// q = dt_max / dt.  For q = M 2^E with 0 <= E < 64 and the mantissa M in [1 + 2^-40,
// 2 - 2^-40], log2 q lies at least 6.5e-13 inside (E, E + 1), while invlogetwo log q is
// within 1.8e-13 of log2 q (invlogetwo is 2.4e-15 relative below 1/ln 2, the logarithm and
// the product within an ulp each, |log2 q| < 64): the truncation is E, and the level E + 1
// is read from the exponent bits.  The fp64 logarithm (GB300: fp64 at 1/64 of the fp32
// rate) is taken only for the other quotients.
__device__ __forceinline__ int timestep_level(double dt, double dt_max) {
  const double q = __ddiv_rn(dt_max, dt);
  const long long b = __double_as_longlong(q);
  const int ebits = (int) ((b >> 52) & 0x7ff);
  const long long mant = b & ((1ll << 52) - 1);
  int l;
  if (b > 0 && ebits >= 1023 && ebits < 1023 + 64 && mant >= (1ll << 12) && mant <= (1ll << 52) - (1ll << 12))
    l = ebits - 1023 + 1;
  else
    l = (int) __dmul_rn(kInvLogTwo, log(q)) + 1;
  return l > 0 ? l : 0;
}

// SphIntegration::Timestep (Courant + acceleration + energy conditions)
__device__ __forceinline__ double particle_timestep(const KdkState& s, const KdkParams& kp, int i, unsigned* status) {
  const double h = s.h[i];
  const double sound = s.keep[kKSound][i];
  const double divv = s.keep[kKDivV][i];
  double ts = __ddiv_rn(__dmul_rn(kp.courant_mult, h), __dadd_rn(__dadd_rn(sound, __dmul_rn(h, fabs(divv))), kSmallDp));
  const double ax = s.keep[kKAX][i], ay = s.keep[kKAY][i], az = s.keep[kKAZ][i];
  const double amag = sqrt(__dadd_rn(__dadd_rn(__dmul_rn(ax, ax), __dmul_rn(ay, ay)), __dmul_rn(az, az)));
  ts = fmin(ts, __dmul_rn(kp.accel_mult, sqrt(__ddiv_rn(h, __dadd_rn(amag, kSmallDp)))));
  if (kp.energy_integration)
    ts = fmin(ts, __dmul_rn(kp.energy_mult, __ddiv_rn(s.u[i], __dadd_rn(fabs(s.keep[kKDudt][i]), 1.0e-20))));
  if (!(ts <= 1.0e20) || !(ts > 0.0)) atomicOr(status, (unsigned) kKdkTimestepInvalid);
  return ts;
}

__device__ __forceinline__ unsigned long long dbits(double x) { return (unsigned long long) __double_as_longlong(x); }

__global__ void k_kdk_begin(KdkGlobal* g) {
  if (threadIdx.x | blockIdx.x) return;
  g->n += 1;
  g->Nsteps += 1;
  g->t = __dadd_rn(g->t, g->timestep);
}

__global__ void k_kdk_advance(KdkState s, KdkParams kp, KdkGlobal* g) {
  const int n = g->n;
  const double t = g->t;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < s.n; i += gridDim.x * blockDim.x) {
    const double dt = __dsub_rn(t, s.tlast[i]);
    double* r[3] = {s.x, s.y, s.z};
    double* v[3] = {s.vx, s.vy, s.vz};
    for (int k = 0; k < 3; k++) {
      const double a0 = s.a0[k][i], v0 = s.v0[k][i];
      r[k][i] = __dadd_rn(__dadd_rn(s.r0[k][i], __dmul_rn(v0, dt)), __dmul_rn(__dmul_rn(__dmul_rn(0.5, a0), dt), dt));
      v[k][i] = __dadd_rn(v0, __dmul_rn(a0, dt));
    }
    if (kp.energy_integration) s.u[i] = __dadd_rn(s.u0[i], __dmul_rn(s.dudt0[i], dt));
    unsigned char f = s.flags[i];
    if (n - s.nlast[i] == s.nstep[i]) f |= kFlagActive; else f &= (unsigned char) ~kFlagActive;
    s.flags[i] = f;
    if (kp.periodic) {
      for (int k = 0; k < 3; k++) {
        if (r[k][i] < kp.boxmin[k]) {
          r[k][i] = __dadd_rn(r[k][i], kp.boxsize[k]);
          s.r0[k][i] = __dadd_rn(s.r0[k][i], kp.boxsize[k]);
        }
        if (r[k][i] > kp.boxmax[k]) {
          r[k][i] = __dsub_rn(r[k][i], kp.boxsize[k]);
          s.r0[k][i] = __dsub_rn(s.r0[k][i], kp.boxsize[k]);
        }
      }
    }
  }
}

// Persistent fields into leaf order after a build; active flags and levels per slot.
// Only what the pass reads of a particle it does not solve: the neighbour fields (h, u and
// the positions come with the tree build's own gather); the solved particles' fields are
// all written by the pass.
__global__ void k_kdk_gather(KdkState s, KdkLeaf l, KdkGlobal* g) {
  unsigned long long act = 0;
  for (int slot = blockIdx.x * blockDim.x + threadIdx.x; slot < l.n; slot += gridDim.x * blockDim.x) {
    const int i = l.id[slot];
#pragma unroll
    for (int q = 0; q < kKeepNeighbour; q++) l.f[q][slot] = s.keep[q][i];
    const unsigned char f = s.flags[i];
    const unsigned char a = f & kFlagActive;
    if (a) s.flags[i] = f | kFlagTouched;
    l.active[slot] = a;
    l.level[slot] = s.level[i];
    l.lvn[slot] = 0;
    act += a;
  }
  for (int o = 16; o > 0; o >>= 1) act += __shfl_xor_sync(0xffffffffu, act, o);
  if ((threadIdx.x & 31) == 0 && act) atomicAdd(&g->active_updates, act);
}

// Solved fields back to input order; levelneib = max(old (0 if active), neighbours).
__global__ void k_kdk_scatter(KdkState s, KdkLeaf l) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < l.n; i += gridDim.x * blockDim.x) {
    const int slot = l.slot_of[i];
#pragma unroll
    for (int q = 0; q < kKeep; q++) s.keep[q][i] = l.f[q][slot];
    s.h[i] = l.h[slot];
    s.u[i] = l.u[slot];
    const int base = l.active[slot] ? 0 : s.levelneib[i];
    s.levelneib[i] = max(base, l.lvn[slot]);
    s.flags[i] &= (unsigned char) ~kFlagTouched;
  }
}

// Later passes of a step reuse the leaf-order fields in place: only the active flags, levels
// and the levelneib accumulators are refreshed.
__global__ void k_kdk_refresh(KdkState s, KdkLeaf l, KdkGlobal* g) {
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&g->repeat_passes, 1ull);
  unsigned long long act = 0;
  for (int slot = blockIdx.x * blockDim.x + threadIdx.x; slot < l.n; slot += gridDim.x * blockDim.x) {
    const int i = l.id[slot];
    const unsigned char f = s.flags[i];
    const unsigned char a = f & kFlagActive;
    if (a) s.flags[i] = f | kFlagTouched;
    l.active[slot] = a;
    l.level[slot] = s.level[i];
    l.lvn[slot] = 0;
    act += a;
  }
  for (int o = 16; o > 0; o >>= 1) act += __shfl_xor_sync(0xffffffffu, act, o);
  if ((threadIdx.x & 31) == 0 && act) atomicAdd(&g->active_updates, act);
}

// levelneib only (what CheckTimesteps reads between passes).
__global__ void k_kdk_scatter_lvn(KdkState s, KdkLeaf l) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < l.n; i += gridDim.x * blockDim.x) {
    const int slot = l.slot_of[i];
    const int base = l.active[slot] ? 0 : s.levelneib[i];
    s.levelneib[i] = max(base, l.lvn[slot]);
  }
}

// Solved fields back to input order, once per step after the last pass.
// Particles solved in some pass of the step get all their fields back; the others only
// the pressure and sound speed the thermal update recomputed (their other fields are
// unchanged, and the leaf-order copies of those were not gathered).
__global__ void k_kdk_scatter_fields(KdkState s, KdkLeaf l) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < l.n; i += gridDim.x * blockDim.x) {
    const int slot = l.slot_of[i];
    const unsigned char f = s.flags[i];
    if (f & kFlagTouched) {
#pragma unroll
      for (int q = 0; q < kKeep; q++) s.keep[q][i] = l.f[q][slot];
      s.h[i] = l.h[slot];
      s.u[i] = l.u[slot];
      s.flags[i] = f & (unsigned char) ~kFlagTouched;
    } else {
      s.keep[kKPressure][i] = l.f[kKPressure][slot];
      s.keep[kKSound][i] = l.f[kKSound][slot];
    }
  }
}

__global__ void k_kdk_check_reset(KdkGlobal* g) {
  if (threadIdx.x | blockIdx.x) return;
  g->activecount = 0;
}

__global__ void k_kdk_check(KdkState s, KdkParams kp, KdkGlobal* g) {
  const int n = g->n, level_step = g->level_step;
  int cnt = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < s.n; i += gridDim.x * blockDim.x) {
    unsigned char f = s.flags[i] & (unsigned char) ~kFlagActive;
    if (kp.nlevels > 1) {
      const int dn = n - s.nlast[i];
      if (dn != s.nstep[i] && s.levelneib[i] - s.level[i] > kp.level_diff_max) {
        const int level_new = s.levelneib[i] - kp.level_diff_max;
        const int nnewstep = pow2i(level_step - level_new);
        if (nnewstep > 0 && dn % nnewstep == 0) {
          if (dn > 0) s.nstep[i] = dn;
          s.level[i] = level_new;
          f |= kFlagActive;
          cnt++;
        }
      }
    }
    s.flags[i] = f;
  }
  for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
  if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(&g->activecount, cnt);
}

__global__ void k_kdk_check_final(KdkGlobal* g) {
  if (threadIdx.x | blockIdx.x) return;
  if (g->activecount > 0) g->status |= kKdkNotSettled;
}

// ---- block timesteps -------------------------------------------------------------------
__global__ void k_bt_prepare(KdkGlobal* g) {
  if (threadIdx.x | blockIdx.x) return;
  g->resync = g->n == g->nresync;
  g->bt_count = 0;
  g->dtmin_bits = dbits(9.9e99);
  g->level_max_new = 0;
  g->nfactor_up = g->nfactor_down = 0;
}

// Phase A: the particles that start a new step (all of them when resyncing) go to a list;
// the levels of the others enter the level_max reduction.  The fp64 timesteps are computed
// over the list (k_bt_a2): GB300 charges an fp64 instruction per warp whatever its active
// lanes, and the particles ending a step are scattered over input order, so computing them
// in place made nearly every warp pay for two divisions, two square roots and a logarithm.
__global__ void k_bt_a(KdkState s, KdkParams kp, KdkGlobal* g) {
  const bool resync = g->resync;
  const int n = g->n;
  const int lane = threadIdx.x & 31;
  int lmax = 0;
  const int stride = gridDim.x * blockDim.x;
  for (int base = blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < s.n; base += stride) {
    const int i = base + lane;
    bool need = false;
    if (i < s.n && (resync || kp.nlevels > 1)) {
      if (resync || n - s.nlast[i] == s.nstep[i]) need = true;
      else lmax = max(lmax, s.level[i]);
    }
    const unsigned m = __ballot_sync(0xffffffffu, need);
    if (m) {
      int at = 0;
      if (lane == 0) at = atomicAdd(&g->bt_count, __popc(m));
      at = __shfl_sync(0xffffffffu, at, 0);
      if (need) s.bt_list[at + __popc(m & ((1u << lane) - 1u))] = i;
    }
  }
  for (int o = 16; o > 0; o >>= 1) lmax = max(lmax, __shfl_xor_sync(0xffffffffu, lmax, o));
  if (lane == 0 && lmax > 0) atomicMax(&g->level_max_new, lmax);
}

// Phase A, listed particles: new timesteps and levels (the list order does not matter: each
// particle's update is its own, and the reductions are a minimum and a maximum).
__global__ void k_bt_a2(KdkState s, KdkParams kp, KdkGlobal* g) {
  const bool resync = g->resync;
  const int n = g->n, level_step = g->level_step, count = g->bt_count;
  const double dt_max = g->dt_max, timestep = g->timestep;
  unsigned long long mbits = dbits(9.9e99);
  int lmax = 0;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < count; k += gridDim.x * blockDim.x) {
    const int i = s.bt_list[k];
    if (resync) {
      const double dt = particle_timestep(s, kp, i, &g->status);
      s.dt_next[i] = dt;
      const unsigned long long b = dbits(dt);
      if (b < mbits) mbits = b;
      continue;
    }
    // n - nlast == nstep here (the listing condition)
    if (s.nstep[i] != pow2i(level_step - s.level[i])) {
      // timestep reduced by CheckTimesteps (Saitoh & Makino)
      const double dt = particle_timestep(s, kp, i, &g->status);
      const int level = max(timestep_level(dt, dt_max), s.levelneib[i] - kp.level_diff_max);
      s.level[i] = max(s.level[i], level);
      s.levelneib[i] = s.level[i];
      s.nlast[i] = n;
      s.nstep[i] = pow2i(level_step - s.level[i]);
      s.dt_next[i] = __dmul_rn((double) s.nstep[i], timestep);
      s.flags[i] |= kFlagEndStep;
    } else {
      const int nstep = s.nstep[i], last_level = s.level[i];
      const double dt = particle_timestep(s, kp, i, &g->status);
      const int level = max(timestep_level(dt, dt_max), s.levelneib[i] - kp.level_diff_max);
      int nl;
      if (level < last_level && last_level > 1 && n % (2 * nstep) == 0) nl = last_level - 1;
      else if (level > last_level) nl = level;
      else nl = last_level;
      s.level[i] = nl;
      s.levelneib[i] = level;
      s.nlast[i] = n;
      s.nstep[i] = pow2i(level_step - nl);
      s.dt_next[i] = __dmul_rn((double) s.nstep[i], timestep);
      s.flags[i] |= kFlagEndStep;
    }
    lmax = max(lmax, s.level[i]);
  }
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long ob = __shfl_xor_sync(0xffffffffu, mbits, o);
    if (ob < mbits) mbits = ob;
    lmax = max(lmax, __shfl_xor_sync(0xffffffffu, lmax, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMin(&g->dtmin_bits, mbits);
    atomicMax(&g->level_max_new, lmax);
  }
}

// Phase B: the integer-time state.
__global__ void k_bt_b(KdkParams kp, KdkGlobal* g) {
  if (threadIdx.x | blockIdx.x) return;
  if (kp.nlevels == 1) {
    if (!g->resync) return;
    g->n = 0;
    g->level_max = 0;
    g->level_step = 0;
    g->nresync = 1;
    g->timestep = __longlong_as_double((long long) g->dtmin_bits);
    g->timestep_old = g->timestep;
    return;
  }
  if (g->resync) {
    g->n = 0;
    const double dtmin = __longlong_as_double((long long) g->dtmin_bits);
    g->timestep = dtmin;
    g->level_max = kp.nlevels - 1;
    g->level_step = g->level_max;
    g->dt_max = __dmul_rn(dtmin, (double) pow2i(g->level_max));
    g->timestep_old = dtmin;
    g->nresync = pow2i(g->level_step);
    g->timestep = __ddiv_rn(g->dt_max, (double) g->nresync);
    return;
  }
  const int level_max_old = g->level_max;
  const int lm = g->level_max_new;
  const int istep = pow2i(g->level_step - level_max_old + 1);
  int level_max;
  if (lm > level_max_old) {
    const int nf = pow2i(lm - level_max_old);
    g->n *= nf;
    g->nfactor_up = nf;
    level_max = lm;
  } else if (lm <= level_max_old - 1 && level_max_old > 1 && istep > 0 && g->n % istep == 0) {
    level_max = level_max_old - 1;
    const int nf = pow2i(level_max_old - level_max);
    g->n /= nf;
    g->nfactor_down = nf;
  } else {
    level_max = level_max_old;
  }
  g->level_max = level_max;
  g->level_step = level_max;
  g->nresync = pow2i(g->level_step);
  g->timestep = __ddiv_rn(g->dt_max, (double) g->nresync);
}

// Phase C: levels after resynchronisation, or the rescaled integer steps.
__global__ void k_bt_c(KdkState s, KdkParams kp, KdkGlobal* g) {
  const bool resync = g->resync;
  const int n = g->n, level_step = g->level_step, level_max = g->level_max;
  const int up = g->nfactor_up, down = g->nfactor_down;
  const double dt_max = g->dt_max, ts_old = g->timestep_old;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < s.n; i += gridDim.x * blockDim.x) {
    if (kp.nlevels == 1) {
      if (!resync) continue;
      s.flags[i] |= kFlagEndStep;
      s.level[i] = 0;
      s.levelneib[i] = 0;
      s.nstep[i] = 1;
      s.dt_next[i] = ts_old;
      continue;
    }
    if (resync) {
      const int level = min(timestep_level(s.dt_next[i], dt_max), level_max);
      s.level[i] = level;
      s.levelneib[i] = level;
      s.nstep[i] = pow2i(level_step - level);
      s.nlast[i] = n;
      s.dt_next[i] = __dmul_rn((double) s.nstep[i], ts_old);
      s.flags[i] |= kFlagEndStep;
      continue;
    }
    if (up) { s.nstep[i] *= up; s.nlast[i] *= up; }
    if (down) { s.nlast[i] /= down; s.nstep[i] /= down; }
    if (s.nlast[i] == n) s.nstep[i] = pow2i(level_step - s.level[i]);
  }
}

__global__ void k_kdk_end(KdkState s, KdkParams kp, KdkGlobal* g) {
  const int n = g->n;
  const double t = g->t;
  double* v[3] = {s.vx, s.vy, s.vz};
  double* r[3] = {s.x, s.y, s.z};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < s.n; i += gridDim.x * blockDim.x) {
    if (!(s.flags[i] & kFlagEndStep)) continue;
    const double dt = s.dt[i];
    const double a[3] = {s.keep[kKAX][i], s.keep[kKAY][i], s.keep[kKAZ][i]};
    for (int k = 0; k < 3; k++) {
      v[k][i] = __dadd_rn(v[k][i], __dmul_rn(__dmul_rn(0.5, dt), __dsub_rn(a[k], s.a0[k][i])));
      s.r0[k][i] = r[k][i];
      s.v0[k][i] = v[k][i];
      s.a0[k][i] = a[k];
    }
    if (kp.energy_integration) {
      const double dudt = s.keep[kKDudt][i];
      double u = __dadd_rn(s.u[i], __dmul_rn(__dmul_rn(0.5, __dsub_rn(dudt, s.dudt0[i])), dt));
      if (u <= 0.0) u = __dadd_rn(s.u0[i], __dmul_rn(s.dudt0[i], dt));
      s.u[i] = u;
      s.u0[i] = u;
      s.dudt0[i] = dudt;
    }
    s.nlast[i] = n;
    s.tlast[i] = t;
    s.dt[i] = s.dt_next[i];
    s.dt_next[i] = 0.0;
    s.flags[i] = 0;
  }
}

// Initial state (SphSimulation::PostInitialConditionsSetup, SphSimulation.cpp:409-421).
__global__ void k_kdk_setup_state(KdkState s, KdkGlobal* g) {
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    KdkGlobal z{};
    z.level_step = 1;
    *g = z;
  }
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < s.n; i += gridDim.x * blockDim.x) {
    for (int k = 0; k < 3; k++) s.a0[k][i] = 0.0;
    s.u0[i] = s.u[i];
    s.dudt0[i] = 0.0;
    s.dt[i] = 0.0;
    s.dt_next[i] = 0.0;
    s.tlast[i] = 0.0;
    s.nlast[i] = 0;
    s.nstep[i] = 0;
    s.level[i] = 0;
    s.levelneib[i] = 0;
    s.flags[i] = kFlagActive;
    for (int q = 0; q < kKeep; q++) s.keep[q][i] = 0.0;
  }
}

// After the initial force pass: r0, v0, a0 and no particle active.
__global__ void k_kdk_setup_finish(KdkState s) {
  double* r[3] = {s.x, s.y, s.z};
  double* v[3] = {s.vx, s.vy, s.vz};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < s.n; i += gridDim.x * blockDim.x) {
    for (int k = 0; k < 3; k++) {
      s.r0[k][i] = r[k][i];
      s.v0[k][i] = v[k][i];
      s.a0[k][i] = s.keep[kKAX + k][i];
    }
    s.flags[i] = 0;
  }
}

// Thermal properties of every particle before a force pass (the radiation-step update of
// SphSimulation::MainLoop, SphSimulation.cpp:672-679, with GradhSph::ComputeThermalProperties,
// GradhSph.cpp:335-345): u (isothermal: temp0 / (gamma-1) / mu_bar), sound speed, pressure.
__global__ void k_kdk_thermal(Particles p, SphParams prm) {
  const double gm1 = prm.gamma_eos - 1.0;
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < p.n; s += gridDim.x * blockDim.x) {
    double u = p.u[s];
    if (prm.eos == 1) { u = prm.u_iso; p.u[s] = u; }
    p.sound[s] = prm.eos == 1 ? sqrt(gm1 * u) : sqrt(prm.gamma_eos * gm1 * u);
    p.pressure[s] = gm1 * p.rho[s] * u;
  }
}

__global__ void k_kdk_set_cond(cudaGraphConditionalHandle h, const KdkGlobal* g) {
  if (threadIdx.x == 0 && blockIdx.x == 0) cudaGraphSetConditional(h, g->activecount > 0 ? 1u : 0u);
}

int grid_for(int n) { return n < 1 ? 1 : ((n + 255) / 256 < 152 * 8 ? (n + 255) / 256 : 152 * 8); }

}  // namespace

void launch_kdk_begin(KdkGlobal* g, cudaStream_t st) { k_kdk_begin<<<1, 32, 0, st>>>(g); }

void launch_kdk_advance(const KdkState& s, const KdkParams& kp, KdkGlobal* g, cudaStream_t st) {
  k_kdk_advance<<<grid_for(s.n), 256, 0, st>>>(s, kp, g);
}

void launch_kdk_gather(const KdkState& s, const KdkLeaf& l, KdkGlobal* g, cudaStream_t st) {
  k_kdk_gather<<<grid_for(l.n), 256, 0, st>>>(s, l, g);
}

void launch_kdk_refresh(const KdkState& s, const KdkLeaf& l, KdkGlobal* g, cudaStream_t st) {
  k_kdk_refresh<<<grid_for(l.n), 256, 0, st>>>(s, l, g);
}

void launch_kdk_scatter_lvn(const KdkState& s, const KdkLeaf& l, cudaStream_t st) {
  k_kdk_scatter_lvn<<<grid_for(l.n), 256, 0, st>>>(s, l);
}

void launch_kdk_scatter_fields(const KdkState& s, const KdkLeaf& l, cudaStream_t st) {
  k_kdk_scatter_fields<<<grid_for(l.n), 256, 0, st>>>(s, l);
}

void launch_kdk_scatter(const KdkState& s, const KdkLeaf& l, cudaStream_t st) {
  k_kdk_scatter<<<grid_for(l.n), 256, 0, st>>>(s, l);
}

void launch_kdk_check(const KdkState& s, const KdkParams& kp, KdkGlobal* g, bool last_pass, cudaStream_t st) {
  k_kdk_check_reset<<<1, 32, 0, st>>>(g);
  k_kdk_check<<<grid_for(s.n), 256, 0, st>>>(s, kp, g);
  if (last_pass) k_kdk_check_final<<<1, 32, 0, st>>>(g);
}

void launch_kdk_timesteps(const KdkState& s, const KdkParams& kp, KdkGlobal* g, cudaStream_t st) {
  k_bt_prepare<<<1, 32, 0, st>>>(g);
  k_bt_a<<<grid_for(s.n), 256, 0, st>>>(s, kp, g);
  k_bt_a2<<<grid_for(s.n), 256, 0, st>>>(s, kp, g);
  k_bt_b<<<1, 32, 0, st>>>(kp, g);
  k_bt_c<<<grid_for(s.n), 256, 0, st>>>(s, kp, g);
}

void launch_kdk_end(const KdkState& s, const KdkParams& kp, KdkGlobal* g, cudaStream_t st) {
  k_kdk_end<<<grid_for(s.n), 256, 0, st>>>(s, kp, g);
}

void launch_kdk_setup_state(const KdkState& s, KdkGlobal* g, cudaStream_t st) {
  k_kdk_setup_state<<<grid_for(s.n), 256, 0, st>>>(s, g);
}

void launch_kdk_thermal(const Particles& p, const SphParams& prm, cudaStream_t st) {
  k_kdk_thermal<<<grid_for(p.n), 256, 0, st>>>(p, prm);
}

void launch_kdk_set_cond(cudaGraphConditionalHandle h, const KdkGlobal* g, cudaStream_t st) {
  k_kdk_set_cond<<<1, 32, 0, st>>>(h, g);
}

void launch_kdk_setup_finish(const KdkState& s, cudaStream_t st) {
  k_kdk_setup_finish<<<grid_for(s.n), 256, 0, st>>>(s);
}

}  // namespace gsph
