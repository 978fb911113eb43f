// Warp-cooperative walk of the depth-first KD-tree.
//
// The reference walks one leaf cell's interaction lists with a stackless loop over the
// copen/cnext links (src/Tree/Tree.cpp:290-381, :561-617, :627-735).  On the GPU one warp
// owns one leaf cell: each round the warp pops up to 32 cells from a per-warp stack in
// shared memory, each lane decides its cell, opened cells push both children, and
// emitted cells are appended to up to three per-warp lists with ballot/popc compaction.
// The decision for a cell depends only on that cell's geometry, so the visited set and
// every list's membership equal the reference walk's; only the order of the entries
// differs.  When a list fills, the caller's flush consumes it and the walk continues, so
// no interaction list can overflow.
#pragma once
#include "gsph_common.cuh"

namespace gsph {

enum WalkAction : int { kSkip = 0, kOpen = 1, kEmitA = 2, kEmitB = 3, kEmitC = 4 };

struct WarpLists {
  int* a;
  int* b;
  int* c;
  int na, nb, nc;     // warp-uniform counts
  int cap;            // capacity of each list
  // round-robin slicing of list a: keep the k-th emitted entry only if k % mod == sel
  int mod = 1, sel = 0, emitted_a = 0;
};

// Returns false when the stack would overflow (status is then the caller's to set).
// decide(node, int& level) -> WalkAction, called by active lanes only; it reports the
// cell's level (callers whose cell records carry it save a load).
// emit_tag(node, action) -> value stored in the list (lets callers pack extra bits).
template <class Decide, class Tag, class Flush>
__device__ __forceinline__ bool warp_walk_lv(int root, int ltot, int* stack, int stack_cap, WarpLists& L, Decide decide,
                                          Tag emit_tag, Flush flush) {
  const int lane = threadIdx.x & 31;
  const unsigned lt = (1u << lane) - 1u;
  if (lane == 0) stack[0] = root;
  int top = 1;
  __syncwarp();
  while (top > 0) {
    const int take = top < 32 ? top : 32;
    int node = -1;
    if (lane < take) node = stack[top - 1 - lane];
    top -= take;
    __syncwarp();
    int act = kSkip, level = 0;
    if (node >= 0) act = decide(node, level);
    const unsigned mo = __ballot_sync(kFull, act == kOpen);
    const int nopen = __popc(mo);
    if (top + 2 * nopen > stack_cap) return false;
    if (act == kOpen) {
      const int r = __popc(mo & lt);
      stack[top + 2 * r] = c2_of(node, level, ltot);
      stack[top + 2 * r + 1] = node + 1;
    }
    top += 2 * nopen;
    const unsigned me = __ballot_sync(kFull, act == kEmitA);
    bool keep = act == kEmitA;
    if (L.mod > 1) keep = keep && ((L.emitted_a + __popc(me & lt)) % L.mod == L.sel);
    L.emitted_a += __popc(me);
    const unsigned ma = __ballot_sync(kFull, keep);
    const unsigned mb = __ballot_sync(kFull, act == kEmitB);
    const unsigned mc = __ballot_sync(kFull, act == kEmitC);
    if (keep) L.a[L.na + __popc(ma & lt)] = emit_tag(node, act);
    if (act == kEmitB) L.b[L.nb + __popc(mb & lt)] = emit_tag(node, act);
    if (act == kEmitC) L.c[L.nc + __popc(mc & lt)] = emit_tag(node, act);
    L.na += __popc(ma);
    L.nb += __popc(mb);
    L.nc += __popc(mc);
    __syncwarp();
    if (L.na > L.cap - 32 || L.nb > L.cap - 32 || L.nc > L.cap - 32) {
      flush();
      L.na = L.nb = L.nc = 0;
      __syncwarp();
    }
  }
  return true;
}

// The same walk with the level read from cell_level; decide(node, level) -> WalkAction.
template <class Decide, class Tag, class Flush>
__device__ __forceinline__ bool warp_walk(int root, int ltot, const unsigned char* __restrict__ cell_level,
                                          int* stack, int stack_cap, WarpLists& L, Decide decide,
                                          Tag emit_tag, Flush flush) {
  auto decide_lv = [&](int node, int& level) -> int {
    level = cell_level[node];
    return decide(node, level);
  };
  return warp_walk_lv(root, ltot, stack, stack_cap, L, decide_lv, emit_tag, flush);
}

__device__ __forceinline__ bool box_overlap(const double* amin, const double* amax, const double* bmin,
                                            const double* bmax) {
#pragma unroll
  for (int k = 0; k < 3; k++) {
    if (amin[k] > bmax[k]) return false;
    if (bmin[k] > amax[k]) return false;
  }
  return true;
}

}  // namespace gsph
