// Shared device definitions for the GB300 grad-h SPH + KD-tree gravity path.
//
// Layout in HBM (all structure-of-arrays, particles in leaf-cell order after a build):
//   particles  : x y z vx vy vz m u h (fp64), plus solved fields rho invomega zeta
//                hfactor hrangesqd pressure sound and force outputs
//   cells      : depth-first cell ids exactly as the reference KD-tree numbers them
//                (src/Tree/KDTree.cpp:361-433): c1 = c + 1, c2 = c + 2^(ltot-level),
//                cnext = c + 2^(ltot-level+1) - 1; per-cell records below.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace gsph {

constexpr double kInvPi = 0.31830988618379;   // reference constant, src/Headers/Constants.h:63
constexpr double kSmall = 1.0e-20;            // src/Headers/Constants.h:73
constexpr double kBig = 9.9e20;               // src/Headers/Constants.h:72
constexpr double kKernRange = 2.0;            // M4 support, src/Hydrodynamics/M4Kernel.cpp:37-56
constexpr double kKernRangeSqd = 4.0;
constexpr double kGhostRange = 2.5;           // src/Headers/Hydrodynamics.h:52
constexpr double kTwoPi = 6.28318530717959;   // src/Headers/Constants.h:62
constexpr int kWarp = 32;
constexpr unsigned kFull = 0xffffffffu;

// Geometry of one cell as the walks read it (48 bytes + 48 bytes of boxes).
struct CellGeom {
  double rcell[3];
  double rmax;
  double hmax;
  double cdistsqd;
};
struct CellBox {
  double bbmin[3], bbmax[3];
};
// Multipole record: centre of mass, mass and the 5 stored traceless quadrupole terms.
struct CellMoment {
  double r[3];
  double m;
  double q[5];
  double pad;
};

// Static topology of a tree with N particles (depends on N and Nleafmax only).
struct TreeShape {
  int n;          // particles
  int ltot;       // leaf level
  int ncell;      // 2^(ltot+1) - 1
  int nleaf;      // 2^ltot
};

// ---- exact (no-contraction) arithmetic for every comparison that decides membership --
__device__ __forceinline__ double dot3_rn(double x, double y, double z) {
  return __dadd_rn(__dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y)), __dmul_rn(z, z));
}
__device__ __forceinline__ double sq_rn(double x) { return __dmul_rn(x, x); }

__device__ __forceinline__ int c2_of(int c, int level, int ltot) { return c + (1 << (ltot - level)); }
__device__ __forceinline__ int cnext_of(int c, int level, int ltot) {
  return level == ltot ? c + 1 : c + (1 << (ltot - level + 1)) - 1;
}

// Order-preserving map of an IEEE double onto uint64.
__device__ __forceinline__ unsigned long long dkey(double v) {
  unsigned long long u = (unsigned long long) __double_as_longlong(v);
  return (u & 0x8000000000000000ull) ? ~u : (u | 0x8000000000000000ull);
}
__device__ __forceinline__ double dkey_inv(unsigned long long k) {
  unsigned long long u = (k & 0x8000000000000000ull) ? (k & 0x7fffffffffffffffull) : ~k;
  return __longlong_as_double((long long) u);
}

// ---- M4 kernel, fp64 (src/Headers/SmoothingKernel.h:131-240) --------------------------
__device__ __forceinline__ double m4_w0(double s) {
  if (s < 1.0) return kInvPi * (1.0 - 1.5 * s * s + 0.75 * s * s * s);
  if (s < 2.0) { const double t = 2.0 - s; return 0.25 * kInvPi * (t * t * t); }
  return 0.0;
}
__device__ __forceinline__ double m4_w1(double s) {
  if (s < 1.0) return kInvPi * (-3.0 * s + 2.25 * s * s);
  if (s < 2.0) return -0.75 * kInvPi * (2.0 - s) * (2.0 - s);
  return 0.0;
}
__device__ __forceinline__ double m4_womega(double s) {
  if (s < 1.0) return kInvPi * (-3.0 + 7.5 * s * s - 4.5 * s * s * s);
  if (s < 2.0) return kInvPi * (-6.0 + 12.0 * s - 7.5 * s * s + 1.5 * s * s * s);
  return 0.0;
}
__device__ __forceinline__ double m4_wzeta(double s) {
  const double s2 = s * s;
  if (s < 1.0) return 1.4 - 2.0 * s2 + 1.5 * s2 * s2 - 0.6 * s2 * s2 * s;
  if (s < 2.0) return 1.6 - 4.0 * s2 + 4.0 * s2 * s - 1.5 * s2 * s2 + 0.2 * s2 * s2 * s;
  return 0.0;
}
__device__ __forceinline__ double m4_wgrav(double s) {
  const double s2 = s * s;
  if (s < 1.0) return 1.333333333333333333333 * s - 1.2 * s2 * s + 0.5 * s2 * s2;
  if (s < 2.0)
    return 2.6666666666666666667 * s - 3.0 * s2 + 1.2 * s2 * s - 0.166666666666666666667 * s2 * s2 -
           0.06666666666666666667 / s2;
  return 1.0 / s2;
}
// wgrav and wpot with 1/s supplied by the caller (h / |r| from the pair's 1/|r|): the
// pair loop then divides once per pair instead of up to five times.
__device__ __forceinline__ double m4_wgrav_r(double s, double inv_s) {
  const double s2 = s * s;
  if (s < 1.0) return 1.333333333333333333333 * s - 1.2 * s2 * s + 0.5 * s2 * s2;
  const double inv_s2 = inv_s * inv_s;
  if (s < 2.0)
    return 2.6666666666666666667 * s - 3.0 * s2 + 1.2 * s2 * s - 0.166666666666666666667 * s2 * s2 -
           0.06666666666666666667 * inv_s2;
  return inv_s2;
}
__device__ __forceinline__ double m4_wpot_r(double s, double inv_s) {
  const double s2 = s * s;
  if (s < 1.0) return 1.4 - 0.666666666666666666666666 * s2 + 0.3 * s2 * s2 - 0.1 * s2 * s2 * s;
  if (s < 2.0)
    return -(1.0 / 15.0) * inv_s + 1.6 - 1.33333333333333333333333333 * s2 + s2 * s - 0.3 * s2 * s2 +
           (1.0 / 30.0) * s2 * s2 * s;
  return inv_s;
}
__device__ __forceinline__ double m4_wpot(double s) {
  const double s2 = s * s;
  if (s < 1.0) return 1.4 - 0.666666666666666666666666 * s2 + 0.3 * s2 * s2 - 0.1 * s2 * s2 * s;
  if (s < 2.0)
    return -1.0 / (15.0 * s) + 1.6 - 1.33333333333333333333333333 * s2 + s2 * s - 0.3 * s2 * s2 +
           (1.0 / 30.0) * s2 * s2 * s;
  return 1.0 / s;
}

// ---- M4 kernel, fp32 (mixed form) ------------------------------------------------------
__device__ __forceinline__ float m4f_w0(float s) {
  if (s < 1.0f) return (float) kInvPi * (1.0f - 1.5f * s * s + 0.75f * s * s * s);
  if (s < 2.0f) { const float t = 2.0f - s; return 0.25f * (float) kInvPi * (t * t * t); }
  return 0.0f;
}
__device__ __forceinline__ float m4f_w1(float s) {
  if (s < 1.0f) return (float) kInvPi * (-3.0f * s + 2.25f * s * s);
  if (s < 2.0f) return -0.75f * (float) kInvPi * (2.0f - s) * (2.0f - s);
  return 0.0f;
}
__device__ __forceinline__ float m4f_womega(float s) {
  if (s < 1.0f) return (float) kInvPi * (-3.0f + 7.5f * s * s - 4.5f * s * s * s);
  if (s < 2.0f) return (float) kInvPi * (-6.0f + 12.0f * s - 7.5f * s * s + 1.5f * s * s * s);
  return 0.0f;
}
__device__ __forceinline__ float m4f_wzeta(float s) {
  const float s2 = s * s;
  if (s < 1.0f) return 1.4f - 2.0f * s2 + 1.5f * s2 * s2 - 0.6f * s2 * s2 * s;
  if (s < 2.0f) return 1.6f - 4.0f * s2 + 4.0f * s2 * s - 1.5f * s2 * s2 + 0.2f * s2 * s2 * s;
  return 0.0f;
}
// Softened force kernel times 1/r for r >= 2h is 1/s^2; the callers handle s >= 2 apart.
__device__ __forceinline__ float m4f_wgrav(float s) {
  const float s2 = s * s;
  if (s < 1.0f) return 1.3333333333f * s - 1.2f * s2 * s + 0.5f * s2 * s2;
  if (s < 2.0f)
    return 2.6666666667f * s - 3.0f * s2 + 1.2f * s2 * s - 0.1666666667f * s2 * s2 - 0.0666666667f / s2;
  return 1.0f / s2;
}
__device__ __forceinline__ float m4f_wpot(float s) {
  const float s2 = s * s;
  if (s < 1.0f) return 1.4f - 0.6666666667f * s2 + 0.3f * s2 * s2 - 0.1f * s2 * s2 * s;
  if (s < 2.0f)
    return -1.0f / (15.0f * s) + 1.6f - 1.3333333333f * s2 + s2 * s - 0.3f * s2 * s2 +
           (1.0f / 30.0f) * s2 * s2 * s;
  return 1.0f / s;
}
// The same two functions with 1/s supplied by the caller (h / |r| from the pair's rsqrt),
// so the pair loops carry no division.
__device__ __forceinline__ float m4f_wgrav_r(float s, float inv_s) {
  const float s2 = s * s;
  if (s < 1.0f) return 1.3333333333f * s - 1.2f * s2 * s + 0.5f * s2 * s2;
  const float inv_s2 = inv_s * inv_s;
  if (s < 2.0f)
    return 2.6666666667f * s - 3.0f * s2 + 1.2f * s2 * s - 0.1666666667f * s2 * s2 - 0.0666666667f * inv_s2;
  return inv_s2;
}
__device__ __forceinline__ float m4f_wpot_r(float s, float inv_s) {
  const float s2 = s * s;
  if (s < 1.0f) return 1.4f - 0.6666666667f * s2 + 0.3f * s2 * s2 - 0.1f * s2 * s2 * s;
  if (s < 2.0f)
    return -(1.0f / 15.0f) * inv_s + 1.6f - 1.3333333333f * s2 + s2 * s - 0.3f * s2 * s2 +
           (1.0f / 30.0f) * s2 * s2 * s;
  return inv_s;
}

// w0, womega and wzeta of one s together (the three sums of the h iteration), one branch.
__device__ __forceinline__ void m4f_w0_omega_zeta(float s, float& w0, float& wom, float& wze) {
  const float s2 = s * s;
  if (s < 1.0f) {
    w0 = (float) kInvPi * (1.0f - 1.5f * s2 + 0.75f * s2 * s);
    wom = (float) kInvPi * (-3.0f + 7.5f * s2 - 4.5f * s2 * s);
    wze = 1.4f - 2.0f * s2 + 1.5f * s2 * s2 - 0.6f * s2 * s2 * s;
  } else {
    const float t = 2.0f - s;
    w0 = 0.25f * (float) kInvPi * (t * t * t);
    wom = (float) kInvPi * (-6.0f + 12.0f * s - 7.5f * s2 + 1.5f * s2 * s);
    wze = 1.6f - 4.0f * s2 + 4.0f * s2 * s - 1.5f * s2 * s2 + 0.2f * s2 * s2 * s;
  }
}

// w1, wgrav and wpot of one s together (one branch on the kernel's piecewise range for
// the three functions), with 1/s supplied by the caller.
__device__ __forceinline__ void m4f_w1_grav_pot(float s, float inv_s, float& w1, float& wg, float& wp) {
  const float s2 = s * s;
  if (s < 1.0f) {
    w1 = (float) kInvPi * (-3.0f * s + 2.25f * s2);
    wg = 1.3333333333f * s - 1.2f * s2 * s + 0.5f * s2 * s2;
    wp = 1.4f - 0.6666666667f * s2 + 0.3f * s2 * s2 - 0.1f * s2 * s2 * s;
  } else if (s < 2.0f) {
    const float inv_s2 = inv_s * inv_s;
    w1 = -0.75f * (float) kInvPi * (2.0f - s) * (2.0f - s);
    wg = 2.6666666667f * s - 3.0f * s2 + 1.2f * s2 * s - 0.1666666667f * s2 * s2 - 0.0666666667f * inv_s2;
    wp = -(1.0f / 15.0f) * inv_s + 1.6f - 1.3333333333f * s2 + s2 * s - 0.3f * s2 * s2 +
         (1.0f / 30.0f) * s2 * s2 * s;
  } else {
    w1 = 0.0f;
    wg = inv_s * inv_s;
    wp = inv_s;
  }
}

// ---- status words written by kernels (never trap) --------------------------------------
enum StatusBits : unsigned {
  kStatusStackOverflow = 1u << 0,   // walk stack exceeded its capacity
  kStatusHNotConverged = 1u << 1,   // h-rho iteration exhausted fixed point + bisection
  kStatusRetryLimit = 1u << 2,      // hmax growth retries exhausted
  kStatusBadInput = 1u << 3,        // non-finite or non-positive mass / h
  kStatusPartitionWait = 1u << 4,   // a tree-build partition wait gave up (results invalid)
};

}  // namespace gsph
