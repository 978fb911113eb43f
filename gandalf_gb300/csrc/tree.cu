// KD-tree build, stock and hmax update on the GPU, reproducing the reference tree exactly.
//
// Reference algorithm (src/Tree/KDTree.cpp):
//   * ltot = smallest l with Nleafmax * 2^l >= N; all leaves on level ltot (:321-352)
//   * root box = particle extent +- kernrange*h (:269-280)
//   * a cell splits along the longest side of its inherited (loose) box (:492-498), at the
//     (N/2)-th smallest coordinate: child 1 receives the N/2 smallest (:505-533)
//   * cells are stocked bottom-up; cdistsqd = max(rmax^2, hmax^2) / theta^2 (:807-1083)
//
// GB300 design: the recursion becomes ltot level-synchronous passes over position lists.
// Each particle's index is presorted once per axis on (coordinate key, index) — an LSD
// radix sort in the allocating build, a bitonic network in the allocation-free one (its
// scratch has no room for the radix sort's second buffers) — so every segment's median
// along its split axis sits at position first + n/2 of that axis list.  A pass then
// marks each particle's side and stable-partitions all three lists with one global scan,
// which keeps each child's lists sorted; once the segments are small, one block per
// segment finishes the remaining levels in shared memory.  Particles are never moved
// until the final gather into leaf order.  Stocking runs bottom-up in a few launches, each
// reducing up to seven levels of complete subtrees in shared memory.
#include "gsph_state.cuh"
#include "tree.cuh"

namespace gsph {

namespace {

constexpr int kSortBlock = 2048;       // elements per shared-memory bitonic block
constexpr int kScanBlock = 2048;       // positions per partition block (1024 threads x 2)

__device__ __forceinline__ bool key_gt(unsigned long long ka, int ia, unsigned long long kb, int ib) {
  return ka > kb || (ka == kb && ia > ib);
}

__global__ void k_root_box_init(unsigned long long* rootkey) {
  const int t = threadIdx.x;
  if (t < 3) rootkey[t] = ~0ull;       // minima
  else if (t < 6) rootkey[t] = 0ull;   // maxima
}

// Root box: min(r - 2h), max(r + 2h) per axis (order-independent, exact).
__global__ void k_root_box(const double* __restrict__ x, const double* __restrict__ y,
                           const double* __restrict__ z, const double* __restrict__ h, int n,
                           unsigned long long* rootkey) {
  unsigned long long lo[3] = {~0ull, ~0ull, ~0ull}, hi[3] = {0ull, 0ull, 0ull};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double hh = __dmul_rn(kKernRange, h[i]);
    const double c[3] = {x[i], y[i], z[i]};
#pragma unroll
    for (int k = 0; k < 3; k++) {
      lo[k] = min(lo[k], dkey(__dsub_rn(c[k], hh)));
      hi[k] = max(hi[k], dkey(__dadd_rn(c[k], hh)));
    }
  }
#pragma unroll
  for (int k = 0; k < 3; k++) {
    for (int o = 16; o > 0; o >>= 1) {
      lo[k] = min(lo[k], __shfl_xor_sync(kFull, lo[k], o));
      hi[k] = max(hi[k], __shfl_xor_sync(kFull, hi[k], o));
    }
  }
  if ((threadIdx.x & 31) == 0) {
    for (int k = 0; k < 3; k++) {
      atomicMin(&rootkey[k], lo[k]);
      atomicMax(&rootkey[3 + k], hi[k]);
    }
  }
}

__global__ void k_root_box_store(const unsigned long long* rootkey, double* ibox) {
  const int t = threadIdx.x;
  if (t < 6) ibox[t] = dkey_inv(rootkey[t]);   // ibox[0..2] = min, [3..5] = max
}

__global__ void k_sort_init(const double* __restrict__ x, const double* __restrict__ y,
                            const double* __restrict__ z, int n, int P, SortArrays s) {
  const int a = blockIdx.y;
  const double* c = a == 0 ? x : (a == 1 ? y : z);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P; i += gridDim.x * blockDim.x) {
    s.key[a][i] = i < n ? dkey(c[i]) : ~0ull;
    s.idx[a][i] = i;
  }
}

// Bitonic stages with strides <= kSortBlock/2 inside shared memory.
__global__ void __launch_bounds__(kSortBlock / 2) k_bitonic_smem(SortArrays s, int kmin, int kmax, int jmax) {
  __shared__ unsigned long long sk[kSortBlock];
  __shared__ int si[kSortBlock];
  const int a = blockIdx.y;
  const int base = blockIdx.x * kSortBlock;
  unsigned long long* key = s.key[a];
  int* idx = s.idx[a];
  for (int t = threadIdx.x; t < kSortBlock; t += blockDim.x) { sk[t] = key[base + t]; si[t] = idx[base + t]; }
  for (int k = kmin; k <= kmax; k <<= 1) {
    for (int j = min(k >> 1, jmax); j > 0; j >>= 1) {
      __syncthreads();
      const int t = threadIdx.x;
      const int i = 2 * j * (t / j) + (t % j);
      const int l = i + j;
      const bool asc = ((base + i) & k) == 0;
      const unsigned long long ki = sk[i], kl = sk[l];
      const int ii = si[i], il = si[l];
      if (key_gt(ki, ii, kl, il) == asc) { sk[i] = kl; sk[l] = ki; si[i] = il; si[l] = ii; }
    }
  }
  __syncthreads();
  for (int t = threadIdx.x; t < kSortBlock; t += blockDim.x) { key[base + t] = sk[t]; idx[base + t] = si[t]; }
}

__global__ void k_bitonic_global(SortArrays s, int P, int k, int j) {
  const int a = blockIdx.y;
  unsigned long long* key = s.key[a];
  int* idx = s.idx[a];
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < P / 2; t += gridDim.x * blockDim.x) {
    const int i = 2 * j * (t / j) + (t % j);
    const int l = i + j;
    const bool asc = (i & k) == 0;
    const unsigned long long ki = key[i], kl = key[l];
    const int ii = idx[i], il = idx[l];
    if (key_gt(ki, ii, kl, il) == asc) { key[i] = kl; key[l] = ki; idx[i] = il; idx[l] = ii; }
  }
}


// ---- LSD radix sort of the (key, index) lists ------------------------------------------
// Eight passes of 8-bit digits; each pass is stable, so equal keys keep ascending index
// order and the result is the order of (key, index), as the bitonic network gives.  The
// three axes are sorted together (blockIdx.y).  Per pass: per-tile digit histograms,
// per-digit prefix over tiles, and a stable scatter in which each tile ranks its elements
// round by round (256 consecutive elements per round: warp match for the rank inside a
// warp, per-warp digit counts in shared memory for the rank across warps).
constexpr int kRadixTile = 4096;           // elements per tile (256 threads x 16 rounds)
constexpr int kRadixRounds = kRadixTile / 256;

// Axis selection with constant indices, so the argument arrays stay in parameter space.
template <class T>
__device__ __forceinline__ T pick3(const T (&v)[3], int a) { return a == 0 ? v[0] : (a == 1 ? v[1] : v[2]); }

__global__ void __launch_bounds__(256) k_radix_hist(RadixArgs r, int shift) {
  __shared__ unsigned cnt[256];
  const int a = blockIdx.y, b = blockIdx.x;
  cnt[threadIdx.x] = 0;
  __syncthreads();
  const unsigned long long* key = pick3(r.src_key, a);
  const int base = b * kRadixTile;
  for (int q = 0; q < kRadixRounds; q++) {
    const int i = base + q * 256 + threadIdx.x;
    if (i < r.n) atomicAdd(&cnt[(unsigned) (key[i] >> shift) & 255u], 1u);
  }
  __syncthreads();
  r.hist[((size_t) a * 256 + threadIdx.x) * r.ntiles + b] = (int) cnt[threadIdx.x];
}

// Exclusive prefix over the tiles of one digit; the digit's total goes to tot.
__device__ __forceinline__ int block_exscan(int v, int* ws, int& total);

__global__ void __launch_bounds__(1024) k_radix_scan(RadixArgs r) {
  __shared__ int ws[33];
  const int a = blockIdx.y, d = blockIdx.x;
  int* h = r.hist + ((size_t) a * 256 + d) * r.ntiles;
  int carry = 0;
  for (int c0 = 0; c0 < r.ntiles; c0 += 1024) {
    const int i = c0 + threadIdx.x;
    const int v = i < r.ntiles ? h[i] : 0;
    int total;
    const int ex = block_exscan(v, ws, total);   // warp shuffles, three barriers
    if (i < r.ntiles) h[i] = carry + ex;
    carry += total;
  }
  if (threadIdx.x == 0) r.tot[a * 256 + d] = carry;
}

// Lanes of the warp holding the same 8-bit digit as this lane (valid lanes only): eight
// ballots, one per digit bit (a warp match waits on the MIO pipe: 24 short-scoreboard
// stalls per issued instruction in this kernel).
__device__ __forceinline__ unsigned digit_peers(unsigned dig, bool valid) {
  unsigned peers = __ballot_sync(kFull, valid);
#pragma unroll
  for (int b = 0; b < 8; b++) {
    const bool on = (dig >> b) & 1u;
    const unsigned m = __ballot_sync(kFull, on);
    peers &= on ? m : ~m;
  }
  return peers;
}

// Inclusive scan of one int per thread over a 256-thread block (warp shuffles, two barriers).
__device__ __forceinline__ int scan256_inclusive(int v, int* wsum) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(kFull, v, o);
    if (lane >= o) v += y;
  }
  if (lane == 31) wsum[w] = v;
  __syncthreads();
  int add = 0;
  for (int q = 0; q < w; q++) add += wsum[q];
  __syncthreads();
  return v + add;
}

// Stable scatter of one tile: warp w owns the tile's elements [w * 512, (w + 1) * 512) in
// rounds of 32 (kept in registers).  Pass 1 counts each digit per warp (warp match: the
// lowest lane of each equal-digit group adds the group's size); the block turns the counts
// into per-warp offsets inside the tile's digit-sorted order; pass 2 places each element in
// shared memory at its warp's running offset plus its rank among the equal digits of its
// round; the tile is then written out in that order, so consecutive threads store
// consecutive positions of each digit's run (coalesced) instead of one 8-byte key and one
// 4-byte index per element scattered over 256 runs.  The element order within a digit is
// the tile order.
constexpr int kRadixWarps = 8;
constexpr int kRadixPerWarp = kRadixTile / kRadixWarps;   // 512
constexpr int kRadixWarpRounds = kRadixPerWarp / 32;      // 16
constexpr size_t kRadixScatterSmem = (size_t) kRadixTile * (sizeof(unsigned long long) + sizeof(int));

__global__ void __launch_bounds__(256) k_radix_scatter(RadixArgs r, int shift) {
  extern __shared__ unsigned long long s_key[];             // kRadixTile keys, then kRadixTile indices
  int* s_idx = reinterpret_cast<int*>(s_key + kRadixTile);
  __shared__ int woff[kRadixWarps][256];   // per-warp digit counts, then offsets in the tile order
  __shared__ int wsum[kRadixWarps];
  __shared__ int dglob[256];                // output position of the tile's first element of each digit
  const int a = blockIdx.y, b = blockIdx.x;
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  for (int d = tid; d < kRadixWarps * 256; d += 256) (&woff[0][0])[d] = 0;
  const unsigned long long* key = pick3(r.src_key, a);
  const int* idx = pick3(r.src_idx, a);
  unsigned long long* okey = pick3(r.dst_key, a);
  int* oidx = pick3(r.dst_idx, a);
  const unsigned lt = (1u << lane) - 1u;
  const int tile0 = b * kRadixTile;
  const int ntile = min(kRadixTile, r.n - tile0);
  const int base = tile0 + w * kRadixPerWarp + lane;
  // exclusive scan of the digit totals (over all tiles)
  const int tot = r.tot[a * 256 + tid];
  const int dstart = scan256_inclusive(tot, wsum) - tot + r.hist[((size_t) a * 256 + tid) * r.ntiles + b];
  // pass 1: per-warp digit counts (the keys are read again in pass 2, from L2)
#pragma unroll 2
  for (int q = 0; q < kRadixWarpRounds; q++) {
    const int i = base + 32 * q;
    const bool valid = i < r.n;
    const unsigned dig = valid ? (unsigned) (key[i] >> shift) & 255u : 0u;
    const unsigned peers = digit_peers(dig, valid);
    if (valid && (peers & lt) == 0u) woff[w][dig] += __popc(peers);
    __syncwarp();
  }
  __syncthreads();
  // the tile's digit counts, their exclusive scan (local digit starts), per-warp offsets
  int cnt = 0;
  for (int v = 0; v < kRadixWarps; v++) cnt += woff[v][tid];
  {
    const int lstart = scan256_inclusive(cnt, wsum) - cnt;
    dglob[tid] = dstart - lstart;
    int run = lstart;
    for (int v = 0; v < kRadixWarps; v++) {
      const int c = woff[v][tid];
      woff[v][tid] = run;
      run += c;
    }
  }
  __syncthreads();
  // pass 2: placement in the tile's digit-sorted order
#pragma unroll
  for (int q = 0; q < kRadixWarpRounds; q++) {
    const int i = base + 32 * q;
    const bool valid = i < r.n;
    const unsigned long long kk = valid ? key[i] : 0ull;
    const unsigned dig = (unsigned) (kk >> shift) & 255u;
    const unsigned peers = digit_peers(dig, valid);
    if (valid) {
      const int pos = woff[w][dig] + __popc(peers & lt);
      s_key[pos] = kk;
      s_idx[pos] = idx[i];
    }
    __syncwarp();
    if (valid && (peers & lt) == 0u) woff[w][dig] += __popc(peers);
    __syncwarp();
  }
  __syncthreads();
  // write-out: position i of the tile order goes to dglob[digit] + i
  for (int i = tid; i < ntile; i += 256) {
    const unsigned long long kk = s_key[i];
    const int pos = dglob[(unsigned) (kk >> shift) & 255u] + i;
    okey[pos] = kk;
    oidx[pos] = s_idx[i];
  }
}

// The radix passes sort on the top kRadixSkipBits.. bits of the keys only (six byte passes
// instead of eight); elements whose keys agree in those bits keep their index order, and
// this pass puts each run of such elements into (full key, index) order.  For coordinates
// the runs are rare (a few per axis among a million random positions) and short; equal full
// keys (lattice positions) are already in index order and cost one comparison each.
constexpr int kRadixSkipBits = 16;

__global__ void k_radix_fixup(SortArrays s, int n) {
  const int a = blockIdx.y;
  unsigned long long* key = pick3(s.key, a);
  int* idx = pick3(s.idx, a);
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    const unsigned long long hj = key[j] >> kRadixSkipBits;
    // a run starts at j when it differs from its left neighbour and equals its right one
    if (j > 0 && (key[j - 1] >> kRadixSkipBits) == hj) continue;
    if (j + 1 >= n || (key[j + 1] >> kRadixSkipBits) != hj) continue;
    int end = j + 1;
    while (end < n && (key[end] >> kRadixSkipBits) == hj) end++;
    // insertion sort of [j, end) by (key, index)
    for (int q = j + 1; q < end; q++) {
      const unsigned long long kq = key[q];
      const int iq = idx[q];
      int r = q - 1;
      while (r >= j && key_gt(key[r], idx[r], kq, iq)) {
        key[r + 1] = key[r];
        idx[r + 1] = idx[r];
        r--;
      }
      key[r + 1] = kq;
      idx[r + 1] = iq;
    }
  }
}

// Segment containing position j on level l (recursive halving of [0, n)).
__device__ __forceinline__ int seg_of(int j, int n, int l, int& first, int& cnt) {
  int s = 0, f = 0, c = n;
  for (int lev = 0; lev < l; lev++) {
    const int half = c >> 1;
    if (j < f + half) { s = 2 * s; c = half; }
    else { s = 2 * s + 1; f += half; c -= half; }
  }
  first = f; cnt = c;
  return s;
}

// One thread per segment of level l: split axis, median coordinate, child boxes.
__global__ void k_split_prepare(int l, BuildLists cur, const double* __restrict__ x,
                                const double* __restrict__ y, const double* __restrict__ z,
                                const int* __restrict__ heap_first, const int* __restrict__ heap_n,
                                double* ibox, unsigned char* seg_axis) {
  const int nseg = 1 << l;
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nseg) return;
  const int hidx = nseg - 1 + s;
  const int first = heap_first[hidx], cnt = heap_n[hidx];
  double bmin[3], bmax[3];
  for (int k = 0; k < 3; k++) { bmin[k] = ibox[6 * hidx + k]; bmax[k] = ibox[6 * hidx + 3 + k]; }
  int kd = 0;
  double rkmax = 0.0;
  for (int k = 0; k < 3; k++) {
    const double ext = __dsub_rn(bmax[k], bmin[k]);
    if (ext > rkmax) { rkmax = ext; kd = k; }
  }
  seg_axis[s] = (unsigned char) kd;
  double rdiv = 0.0;
  if (cnt > 0) {
    const int id = cur.l[kd][first + cnt / 2];
    rdiv = kd == 0 ? x[id] : (kd == 1 ? y[id] : z[id]);
  }
  const int c1 = 2 * hidx + 1, c2 = 2 * hidx + 2;
  for (int k = 0; k < 3; k++) {
    ibox[6 * c1 + k] = bmin[k]; ibox[6 * c1 + 3 + k] = bmax[k];
    ibox[6 * c2 + k] = bmin[k]; ibox[6 * c2 + 3 + k] = bmax[k];
  }
  ibox[6 * c1 + 3 + kd] = rdiv;
  ibox[6 * c2 + kd] = rdiv;
}

__global__ void k_mark_side(int l, int n, BuildLists cur, const unsigned char* __restrict__ seg_axis,
                            unsigned char* side) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    int first, cnt;
    const int s = seg_of(j, n, l, first, cnt);
    const int kd = seg_axis[s];
    side[cur.l[kd][j]] = (unsigned char) (j - first >= (cnt >> 1));
  }
}

__global__ void __launch_bounds__(1024) k_part_count(int n, BuildLists cur, const unsigned char* __restrict__ side,
                                                     int* blocksum, int nb) {
  const int a = blockIdx.y;
  const int base = blockIdx.x * kScanBlock;
  int c = 0;
  for (int t = threadIdx.x; t < kScanBlock; t += blockDim.x) {
    const int j = base + t;
    if (j < n) c += side[cur.l[a][j]];
  }
  c = __reduce_add_sync(kFull, c);
  __shared__ int ws[32];
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x < 32) {
    int v = threadIdx.x < (blockDim.x >> 5) ? ws[threadIdx.x] : 0;
    v = __reduce_add_sync(kFull, v);
    if (threadIdx.x == 0) blocksum[a * nb + blockIdx.x] = v;
  }
}

// Block-wide exclusive scan of one int per thread (1024 threads).
__device__ __forceinline__ int block_exscan(int v, int* ws, int& total) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int inc = v;
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(kFull, inc, o);
    if (lane >= o) inc += y;
  }
  if (lane == 31) ws[w] = inc;
  __syncthreads();
  if (w == 0) {
    int s = lane < (int) (blockDim.x >> 5) ? ws[lane] : 0;
    int si = s;
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(kFull, si, o);
      if (lane >= o) si += y;
    }
    ws[lane] = si - s;
    if (lane == 31) ws[32] = si;
  }
  __syncthreads();
  total = ws[32];
  const int r = ws[w] + inc - v;
  __syncthreads();
  return r;
}

__global__ void __launch_bounds__(1024) k_part_scan(int* blocksum, int nb) {
  __shared__ int ws[33];
  const int a = blockIdx.y;
  int* b = blocksum + a * nb;
  int carry = 0;
  for (int base = 0; base < nb; base += 1024) {
    const int i = base + threadIdx.x;
    const int v = i < nb ? b[i] : 0;
    int total;
    const int ex = block_exscan(v, ws, total);
    if (i < nb) b[i] = carry + ex;
    carry += total;
  }
}

__global__ void __launch_bounds__(1024) k_part_scatter(int l, int n, BuildLists cur, BuildLists nxt,
                                                       const unsigned char* __restrict__ side,
                                                       const int* __restrict__ blocksum, int nb,
                                                       const int* __restrict__ heap_ones_before) {
  __shared__ int ws[33];
  const int a = blockIdx.y;
  const int base = blockIdx.x * kScanBlock;
  const int j0 = base + 2 * threadIdx.x, j1 = j0 + 1;
  const int id0 = j0 < n ? cur.l[a][j0] : -1;
  const int id1 = j1 < n ? cur.l[a][j1] : -1;
  const int f0 = id0 >= 0 ? side[id0] : 0;
  const int f1 = id1 >= 0 ? side[id1] : 0;
  int total;
  const int ex = block_exscan(f0 + f1, ws, total) + blocksum[a * nb + blockIdx.x];
  const int nseg = 1 << l;
  int jj[2] = {j0, j1}, ids[2] = {id0, id1}, ff[2] = {f0, f1}, ee[2] = {ex, ex + f0};
  for (int q = 0; q < 2; q++) {
    if (ids[q] < 0) continue;
    int first, cnt;
    const int s = seg_of(jj[q], n, l, first, cnt);
    const int ob = heap_ones_before[nseg - 1 + s];
    const int ones = ee[q] - ob;                  // ones before j inside the segment
    const int pos = ff[q] ? first + (cnt >> 1) + ones : first + (jj[q] - first) - ones;
    nxt.l[a][pos] = ids[q];
  }
}

// ---- single-pass level partition (the allocating build) ----------------------------------
// One launch per level in place of count + scan + scatter: each block takes one tile
// (kScanBlock positions) of one axis list in the order the blocks start (a ticket, so a
// block only ever waits for blocks already running), counts the tile's second-child marks,
// publishes the count, obtains the count of all earlier tiles of its list by decoupled
// look-back, and scatters.  While it scatters, it also writes the next level's side marks of
// the particles it places into the list of their child's split axis (so the next level needs
// no marking pass).  Tile words: (epoch << 34) | (flag << 32) | count, flag 1 = count of the
// tile alone, 2 = count of the tile and every earlier one.  The epoch advances once per
// launch (the block with the last ticket bumps it and rewinds the ticket counter), so words
// left by earlier launches are never taken for this one's; a wait that runs past its limit
// sets kStatusPartitionWait and continues, and the host reports the error.
constexpr unsigned kLbAggregate = 1u, kLbPrefix = 2u;
constexpr int kLbSpinLimit = 1 << 22;

// Longest side of a box (the split axis rule of KDTree::DivideTreeCell, :492-498).
__device__ __forceinline__ int longest_axis(const double* bmin, const double* bmax) {
  int kd = 0;
  double rkmax = 0.0;
  for (int k = 0; k < 3; k++) {
    const double ext = __dsub_rn(bmax[k], bmin[k]);
    if (ext > rkmax) { rkmax = ext; kd = k; }
  }
  return kd;
}

// k_split_prepare plus the split axes of the children (the next level's segments).
__global__ void k_split_prepare_next(int l, BuildLists cur, const double* __restrict__ x,
                                     const double* __restrict__ y, const double* __restrict__ z,
                                     const int* __restrict__ heap_first, const int* __restrict__ heap_n,
                                     double* ibox, unsigned char* seg_axis, unsigned char* seg_axis_next) {
  const int nseg = 1 << l;
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nseg) return;
  const int hidx = nseg - 1 + s;
  const int first = heap_first[hidx], cnt = heap_n[hidx];
  double bmin[3], bmax[3];
  for (int k = 0; k < 3; k++) { bmin[k] = ibox[6 * hidx + k]; bmax[k] = ibox[6 * hidx + 3 + k]; }
  const int kd = longest_axis(bmin, bmax);
  seg_axis[s] = (unsigned char) kd;
  double rdiv = 0.0;
  if (cnt > 0) {
    const int id = cur.l[kd][first + cnt / 2];
    rdiv = kd == 0 ? x[id] : (kd == 1 ? y[id] : z[id]);
  }
  const int c1 = 2 * hidx + 1, c2 = 2 * hidx + 2;
  double b1[6], b2[6];
  for (int k = 0; k < 3; k++) {
    b1[k] = bmin[k]; b1[3 + k] = bmax[k];
    b2[k] = bmin[k]; b2[3 + k] = bmax[k];
  }
  b1[3 + kd] = rdiv;
  b2[kd] = rdiv;
  for (int k = 0; k < 6; k++) { ibox[6 * c1 + k] = b1[k]; ibox[6 * c2 + k] = b2[k]; }
  seg_axis_next[2 * s] = (unsigned char) longest_axis(b1, b1 + 3);
  seg_axis_next[2 * s + 1] = (unsigned char) longest_axis(b2, b2 + 3);
}

__device__ __forceinline__ unsigned long long lb_word(unsigned epoch, unsigned flag, unsigned v) {
  return ((unsigned long long) epoch << 34) | ((unsigned long long) flag << 32) | (unsigned long long) v;
}

constexpr int kPartThreads = 512, kPartPer = 8;
constexpr int kPartTile = kPartThreads * kPartPer;   // positions per tile

__global__ void __launch_bounds__(kPartThreads) k_part_level(int l, int n, BuildLists cur, BuildLists nxt,
                                                             const unsigned char* __restrict__ side,
                                                             unsigned char* side_next,
                                                             const unsigned char* __restrict__ seg_axis_next,
                                                             const int* __restrict__ heap_ones_before, int nb,
                                                             PartitionState ps) {
  __shared__ int ws[33];
  __shared__ unsigned s_ticket, s_epoch;
  __shared__ int s_before;
  if (threadIdx.x == 0) {
    const unsigned ep = *reinterpret_cast<volatile unsigned*>(ps.epoch);
    __threadfence();
    s_ticket = atomicAdd(ps.ticket, 1u);
    s_epoch = ep & 0x3fffffffu;
  }
  __syncthreads();
  const unsigned ticket = s_ticket, epoch = s_epoch;
  const int total = 3 * nb;
  if ((int) ticket >= total) return;   // cannot happen: one ticket per block of the grid
  // tickets run over the three axes' tiles interleaved, each axis's tiles in order
  const int a = (int) ticket % 3, b = (int) ticket / 3;
  unsigned long long* words = ps.tiles + (size_t) a * nb;
  const int* src = pick3(cur.l, a);
  int* dst = pick3(nxt.l, a);
  // kPartPer consecutive positions a thread
  const int j0 = b * kPartTile + threadIdx.x * kPartPer;
  int ids[kPartPer], f[kPartPer];
  int mine = 0;
#pragma unroll
  for (int q = 0; q < kPartPer; q++) ids[q] = j0 + q < n ? src[j0 + q] : -1;
#pragma unroll
  for (int q = 0; q < kPartPer; q++) {
    f[q] = ids[q] >= 0 ? side[ids[q]] : 0;
    mine += f[q];
  }
  int count;
  const int ex = block_exscan(mine, ws, count);
  // decoupled look-back by warp 0: 32 earlier tiles a probe, summed back to the nearest
  // inclusive prefix
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    unsigned before = 0;
    if (b == 0) {
      if (lane == 0) atomicExch(words, lb_word(epoch, kLbPrefix, (unsigned) count));
    } else {
      if (lane == 0) atomicExch(words + b, lb_word(epoch, kLbAggregate, (unsigned) count));
      int i = b - 1, spins = 0;
      for (;;) {
        const int k = i - lane;
        unsigned flag = kLbPrefix, v = 0;   // before tile 0: an empty prefix
        if (k >= 0) {
          const unsigned long long w = *reinterpret_cast<volatile unsigned long long*>(words + k);
          flag = (unsigned) (w >> 34) == epoch ? (unsigned) (w >> 32) & 3u : 0u;
          v = (unsigned) w;
        }
        if (__any_sync(kFull, flag == 0u)) {   // some earlier tile has not published yet
          if (++spins > kLbSpinLimit) {
            if (lane == 0) atomicOr(ps.status, (unsigned) kStatusPartitionWait);
            break;
          }
          __nanosleep(32);
          continue;
        }
        const unsigned pm = __ballot_sync(kFull, flag == kLbPrefix);
        const int stop = pm ? __ffs(pm) - 1 : 31;   // the nearest inclusive prefix
        before += __reduce_add_sync(kFull, lane <= stop ? v : 0u);
        if (pm) break;
        i -= 32;
        spins = 0;
      }
      if (lane == 0) atomicExch(words + b, lb_word(epoch, kLbPrefix, before + (unsigned) count));
    }
    if (lane == 0) {
      s_before = (int) before;
      if ((int) ticket == total - 1) {
        // every block has its ticket (and has read the epoch before taking it)
        atomicExch(ps.ticket, 0u);
        atomicAdd(ps.epoch, 1u);
      }
    }
  }
  __syncthreads();
  const int nseg = 1 << l;
  int e = s_before + ex;   // ones before this thread's first position, over the whole list
#pragma unroll
  for (int q = 0; q < kPartPer; q++) {
    const int j = j0 + q, id = ids[q];
    if (id >= 0) {
      int first, cnt;
      const int s2 = seg_of(j, n, l, first, cnt);
      const int ones = e - heap_ones_before[nseg - 1 + s2];   // ones before j inside the segment
      const int half = cnt >> 1;
      int pos, cfirst, ccnt;
      if (f[q]) { pos = first + half + ones; cfirst = first + half; ccnt = cnt - half; }
      else { pos = first + (j - first) - ones; cfirst = first; ccnt = half; }
      dst[pos] = id;
      if (side_next && seg_axis_next[2 * s2 + f[q]] == a)
        side_next[id] = (unsigned char) (pos - cfirst >= (ccnt >> 1));
    }
    e += f[q];
  }
}

// ---- the deep levels of a segment in shared memory ---------------------------------------
// Once every segment of a level holds at most kDeepMax particles, one block finishes its
// segment's remaining levels in shared memory: the same split axis, median coordinate,
// child boxes, side marks and stable partitions as the level passes, on 16-bit local ids
// (a particle's position in the segment's x list), with one launch instead of five per
// level.  The block writes the segment's final first list (leaf order) back in place.
constexpr int kDeepMax = 4096;
constexpr int kDeepThreads = 1024;
constexpr int kDeepPer = kDeepMax / kDeepThreads;   // list positions a thread scans

// 86 KB: above the static shared-memory limit, so it is dynamic (one or two blocks an SM)
struct DeepSmem {
  unsigned short l[2][3][kDeepMax];
  int glob[kDeepMax];
  int scan[kDeepMax];
  unsigned char side[kDeepMax];
  unsigned char kd[kDeepMax / 2];
  int ws[33];
};

__global__ void __launch_bounds__(kDeepThreads) k_build_deep(int L0, int ltot, BuildLists cur, int* inv,
                                                            const double* __restrict__ x,
                                                            const double* __restrict__ y,
                                                            const double* __restrict__ z,
                                                            const int* __restrict__ heap_first,
                                                            const int* __restrict__ heap_n, double* ibox) {
  extern __shared__ __align__(16) unsigned char s_deep_raw[];
  DeepSmem& sm = *reinterpret_cast<DeepSmem*>(s_deep_raw);
  auto& s_l = sm.l;
  int* s_glob = sm.glob;
  int* s_scan = sm.scan;
  unsigned char* s_side = sm.side;
  unsigned char* s_kd = sm.kd;
  int* ws = sm.ws;
  const int tid = threadIdx.x;
  const int s0 = blockIdx.x;
  const int h0 = (1 << L0) - 1 + s0;
  const int first = heap_first[h0], cnt = heap_n[h0];
  for (int q = tid; q < cnt; q += kDeepThreads) {
    const int gid = cur.l[0][first + q];
    s_glob[q] = gid;
    s_l[0][0][q] = (unsigned short) q;
    inv[gid] = q;
  }
  __syncthreads();
  for (int a = 1; a < 3; a++)
    for (int q = tid; q < cnt; q += kDeepThreads) s_l[0][a][q] = (unsigned short) inv[cur.l[a][first + q]];
  __syncthreads();
  int cb = 0;
  for (int l = L0; l < ltot; l++) {
    const int d = l - L0, nsub = 1 << d;
    // split axis, median and child boxes of each sub-segment (k_split_prepare)
    for (int q = tid; q < nsub; q += kDeepThreads) {
      const int hidx = (1 << l) - 1 + (s0 << d) + q;
      const int f = heap_first[hidx] - first, c = heap_n[hidx];
      double bmin[3], bmax[3];
      for (int k = 0; k < 3; k++) { bmin[k] = ibox[6 * hidx + k]; bmax[k] = ibox[6 * hidx + 3 + k]; }
      int kd = 0;
      double rkmax = 0.0;
      for (int k = 0; k < 3; k++) {
        const double ext = __dsub_rn(bmax[k], bmin[k]);
        if (ext > rkmax) { rkmax = ext; kd = k; }
      }
      s_kd[q] = (unsigned char) kd;
      double rdiv = 0.0;
      if (c > 0) {
        const int id = s_glob[s_l[cb][kd][f + c / 2]];
        rdiv = kd == 0 ? x[id] : (kd == 1 ? y[id] : z[id]);
      }
      const int c1 = 2 * hidx + 1, c2 = 2 * hidx + 2;
      for (int k = 0; k < 3; k++) {
        ibox[6 * c1 + k] = bmin[k]; ibox[6 * c1 + 3 + k] = bmax[k];
        ibox[6 * c2 + k] = bmin[k]; ibox[6 * c2 + 3 + k] = bmax[k];
      }
      ibox[6 * c1 + 3 + kd] = rdiv;
      ibox[6 * c2 + kd] = rdiv;
    }
    __syncthreads();
    // side marks (k_mark_side)
    for (int q = tid; q < cnt; q += kDeepThreads) {
      int f, c;
      const int sub = seg_of(q, cnt, d, f, c);
      s_side[s_l[cb][s_kd[sub]][q]] = (unsigned char) (q - f >= (c >> 1));
    }
    __syncthreads();
    // stable partition of the three lists inside each sub-segment (k_part_scatter)
    for (int a = 0; a < 3; a++) {
      // positions q0 .. q0 + kDeepPer - 1 of the list, consecutive per thread
      const int q0 = kDeepPer * tid;
      int fl[kDeepPer], sum = 0;
#pragma unroll
      for (int r = 0; r < kDeepPer; r++) {
        fl[r] = q0 + r < cnt ? s_side[s_l[cb][a][q0 + r]] : 0;
        sum += fl[r];
      }
      int total;
      int run = block_exscan(sum, ws, total);
#pragma unroll
      for (int r = 0; r < kDeepPer; r++) {
        if (q0 + r < cnt) s_scan[q0 + r] = run;
        run += fl[r];
      }
      __syncthreads();
#pragma unroll
      for (int r = 0; r < kDeepPer; r++) {
        const int q = q0 + r;
        if (q >= cnt) continue;
        int f, c;
        seg_of(q, cnt, d, f, c);
        const int ones = s_scan[q] - s_scan[f];   // ones before q inside its sub-segment
        const int pos = fl[r] ? f + (c >> 1) + ones : f + (q - f) - ones;
        s_l[cb ^ 1][a][pos] = s_l[cb][a][q];
      }
      __syncthreads();
    }
    cb ^= 1;
  }
  for (int q = tid; q < cnt; q += kDeepThreads) cur.l[0][first + q] = s_glob[s_l[cb][0][q]];
}

__global__ void k_gather_leaf_order(int n, const int* __restrict__ perm, InputArrays in, Particles p,
                                    int* id_out, int* slot_of) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
    const int i = perm[s];
    id_out[s] = i;
    slot_of[i] = s;
    p.x[s] = in.x[i]; p.y[s] = in.y[i]; p.z[s] = in.z[i];
    p.vx[s] = in.vx[i]; p.vy[s] = in.vy[i]; p.vz[s] = in.vz[i];
    p.m[s] = in.m[i]; p.u[s] = in.u[i]; p.h[s] = in.h[i]; p.h0[s] = in.h[i];
  }
}

// ---- stocking (KDTree::StockCellProperties) ------------------------------------------
// Bottom-up over the complete tree (all 2^ltot leaves on level ltot).  One launch takes the
// nodes of one level, kStockBlock consecutive nodes per block (a complete subtree's nodes
// of that level), and reduces up to log2(kStockBlock) levels above them in shared memory;
// the next launch starts from the level where the last one stopped.  1M particles with
// Nleafmax 8 (17 levels): leaves -> level 10 -> level 3 -> root, three launches.  Every
// parent is computed by the lowest threads of its block, so the fp64 arithmetic runs in
// compact warps, with no arrival counters or fences.
constexpr int kStockBlock = 128;
constexpr int kStockLevels = 7;        // log2(kStockBlock)

// min / max of finite doubles through their order-preserving 64-bit keys (dkey): the values
// fmin / fmax give, on the integer pipes — GB300 runs fp64 at 1/64 of the fp32 rate and
// charges each fp64 instruction per warp.  Used by the hmax update (8.4M Evrard sphere:
// 0.86 -> 0.74 ms); in the stock, whose leaf threads already hold 124 registers, the same
// change (with a second-moment quadrupole) made the launch slower and was dropped.
__device__ __forceinline__ double kmin(double a, double b) { return dkey(b) < dkey(a) ? b : a; }
__device__ __forceinline__ double kmax(double a, double b) { return dkey(b) > dkey(a) ? b : a; }

// What a parent's stock needs of each child (KDTree::StockCellProperties, :958-1059).
struct StockNode {
  double bmin[3], bmax[3], hbmin[3], hbmax[3], hmax, m, r[3], q[5];
  int n;
};

// Depth-first id of node k (left to right) of level L.
__device__ __forceinline__ int cell_at(int L, int k, int ltot) {
  int id = 0;
  for (int i = 1; i <= L; i++) id += ((k >> (L - i)) & 1) ? (1 << (ltot - i + 1)) : 1;
  return id;
}

__device__ void finish_geometry(int n, const double* bmin, const double* bmax, double hmax,
                                double theta2, CellGeom& g) {
  if (n > 0) {
    double dr[3];
    for (int k = 0; k < 3; k++) {
      g.rcell[k] = __dmul_rn(0.5, __dadd_rn(bmin[k], bmax[k]));
      dr[k] = __dmul_rn(0.5, __dsub_rn(bmax[k], bmin[k]));
    }
    const double dd = dot3_rn(dr[0], dr[1], dr[2]);
    g.cdistsqd = __ddiv_rn(fmax(dd, __dmul_rn(hmax, hmax)), theta2);
    g.rmax = __dsqrt_rn(dd);
  } else {
    for (int k = 0; k < 3; k++) g.rcell[k] = 0.0;
    g.cdistsqd = kBig;
    g.rmax = 0.0;
  }
  g.hmax = hmax;
}

__device__ void store_cell(const Tree& t, int c, const StockNode& v, const CellGeom& g) {
  t.geom[c] = g;
  CellBox b, hb;
  for (int k = 0; k < 3; k++) {
    b.bbmin[k] = v.bmin[k]; b.bbmax[k] = v.bmax[k]; hb.bbmin[k] = v.hbmin[k]; hb.bbmax[k] = v.hbmax[k];
  }
  t.bb[c] = b;
  t.hbox[c] = hb;
  CellMoment mo;
  for (int k = 0; k < 3; k++) mo.r[k] = v.r[k];
  mo.m = v.m;
  for (int k = 0; k < 5; k++) mo.q[k] = v.q[k];
  mo.pad = 0.0;
  t.mom[c] = mo;
}

__device__ StockNode stock_leaf(const Tree& t, const Particles& p, int c, double theta2) {
  const int first = t.cell_first[c], n = t.cell_n[c];
  StockNode v;
  v.n = n;
  v.m = 0.0; v.hmax = 0.0;
  for (int k = 0; k < 3; k++) {
    v.r[k] = 0.0; v.bmin[k] = kBig; v.bmax[k] = -kBig; v.hbmin[k] = kBig; v.hbmax[k] = -kBig;
  }
  for (int j = 0; j < n; j++) {
    const int s = first + j;
    const double xs[3] = {p.x[s], p.y[s], p.z[s]};
    const double hh = p.h[s], mm = p.m[s];
    v.hmax = fmax(v.hmax, hh);
    v.m += mm;
    const double h2 = __dmul_rn(kKernRange, hh);
    for (int k = 0; k < 3; k++) {
      v.r[k] = fma(mm, xs[k], v.r[k]);
      v.bmin[k] = fmin(v.bmin[k], xs[k]);
      v.bmax[k] = fmax(v.bmax[k], xs[k]);
      v.hbmin[k] = fmin(v.hbmin[k], __dsub_rn(xs[k], h2));
      v.hbmax[k] = fmax(v.hbmax[k], __dadd_rn(xs[k], h2));
    }
  }
  if (v.m > 0.0) {
    const double im = 1.0 / v.m;   // one division for the three components
    for (int k = 0; k < 3; k++) v.r[k] *= im;
  }
  for (int k = 0; k < 5; k++) v.q[k] = 0.0;
  for (int j = 0; j < n; j++) {
    const int s = first + j;
    const double mm = p.m[s];
    const double dx = p.x[s] - v.r[0], dy = p.y[s] - v.r[1], dz = p.z[s] - v.r[2];
    const double drsqd = dx * dx + dy * dy + dz * dz;
    v.q[0] += mm * (3.0 * dx * dx - drsqd);
    v.q[1] += mm * 3.0 * dx * dy;
    v.q[2] += mm * (3.0 * dy * dy - drsqd);
    v.q[3] += mm * 3.0 * dz * dx;
    v.q[4] += mm * 3.0 * dz * dy;
  }
  CellGeom g;
  finish_geometry(n, v.bmin, v.bmax, v.hmax, theta2, g);
  store_cell(t, c, v, g);
  return v;
}

// A stocked cell read back (the input nodes of the upper launches).
__device__ StockNode load_node(const Tree& t, int c) {
  StockNode v;
  const CellBox b = t.bb[c], hb = t.hbox[c];
  const CellMoment mo = t.mom[c];
  for (int k = 0; k < 3; k++) {
    v.bmin[k] = b.bbmin[k]; v.bmax[k] = b.bbmax[k]; v.hbmin[k] = hb.bbmin[k]; v.hbmax[k] = hb.bbmax[k];
    v.r[k] = mo.r[k];
  }
  v.hmax = t.geom[c].hmax;
  v.m = mo.m;
  for (int k = 0; k < 5; k++) v.q[k] = mo.q[k];
  v.n = t.cell_n[c];
  return v;
}

// Parent c from its children a (first) and b (second): boxes and hmax of the non-empty
// children, centre of mass, and the quadrupole moved to the new centre.
__device__ StockNode stock_parent(const Tree& t, int c, const StockNode& a, const StockNode& b, double theta2) {
  StockNode v;
  v.hmax = 0.0;
  for (int k = 0; k < 3; k++) { v.bmin[k] = kBig; v.bmax[k] = -kBig; v.hbmin[k] = kBig; v.hbmax[k] = -kBig; }
  const StockNode* ch[2] = {&a, &b};
  for (int q = 0; q < 2; q++) {
    const StockNode& u = *ch[q];
    if (u.n > 0) {
      for (int k = 0; k < 3; k++) {
        v.bmin[k] = fmin(u.bmin[k], v.bmin[k]);
        v.bmax[k] = fmax(u.bmax[k], v.bmax[k]);
        v.hbmin[k] = fmin(u.hbmin[k], v.hbmin[k]);
        v.hbmax[k] = fmax(u.hbmax[k], v.hbmax[k]);
      }
      v.hmax = fmax(v.hmax, u.hmax);
    }
  }
  v.n = a.n + b.n;
  v.m = a.m + b.m;
  for (int k = 0; k < 3; k++) v.r[k] = 0.0;
  if (v.m > 0.0) {
    const double im = 1.0 / v.m;
    for (int k = 0; k < 3; k++) v.r[k] = (a.m * a.r[k] + b.m * b.r[k]) * im;
  }
  for (int k = 0; k < 5; k++) v.q[k] = 0.0;
  for (int q = 0; q < 2; q++) {
    const StockNode& u = *ch[q];
    if (!(u.m > 0.0)) continue;
    const double dx = u.r[0] - v.r[0], dy = u.r[1] - v.r[1], dz = u.r[2] - v.r[2];
    const double drsqd = dx * dx + dy * dy + dz * dz;
    for (int k = 0; k < 5; k++) v.q[k] += u.q[k];
    v.q[0] += u.m * (3.0 * dx * dx - drsqd);
    v.q[1] += u.m * 3.0 * dx * dy;
    v.q[2] += u.m * (3.0 * dy * dy - drsqd);
    v.q[3] += u.m * 3.0 * dz * dx;
    v.q[4] += u.m * 3.0 * dz * dy;
  }
  CellGeom g;
  finish_geometry(v.n, v.bmin, v.bmax, v.hmax, theta2, g);
  store_cell(t, c, v, g);
  return v;
}

// Shared-memory copy of the nodes of one level (structure of arrays: no bank conflicts).
struct StockSmem {
  double d[21][kStockBlock];
  int n[kStockBlock], cid[kStockBlock];
};

__device__ __forceinline__ void put_node(StockSmem& sm, int i, const StockNode& v, int cid) {
  for (int k = 0; k < 3; k++) {
    sm.d[k][i] = v.bmin[k]; sm.d[3 + k][i] = v.bmax[k]; sm.d[6 + k][i] = v.hbmin[k]; sm.d[9 + k][i] = v.hbmax[k];
    sm.d[13 + k][i] = v.r[k];
  }
  sm.d[12][i] = v.hmax;
  sm.d[16][i] = v.m;
  sm.n[i] = v.n;
  sm.cid[i] = cid;
}

__device__ __forceinline__ StockNode get_node(const StockSmem& sm, const double (*q)[kStockBlock], int i) {
  StockNode v;
  for (int k = 0; k < 3; k++) {
    v.bmin[k] = sm.d[k][i]; v.bmax[k] = sm.d[3 + k][i]; v.hbmin[k] = sm.d[6 + k][i]; v.hbmax[k] = sm.d[9 + k][i];
    v.r[k] = sm.d[13 + k][i];
  }
  v.hmax = sm.d[12][i];
  v.m = sm.d[16][i];
  for (int k = 0; k < 5; k++) v.q[k] = q[k][i];
  v.n = sm.n[i];
  return v;
}

// Nodes of level Lin (leaves when Lin == ltot) -> stocked cells up to level Lout.
__global__ void __launch_bounds__(kStockBlock) k_stock(Tree t, Particles p, double theta2, int Lin, int Lout) {
  __shared__ StockSmem sm;
  __shared__ double sq[5][kStockBlock];   // the quadrupole terms
  const int tid = threadIdx.x;
  const int k = blockIdx.x * blockDim.x + tid;   // node of level Lin
  StockNode v;
  int cid;
  if (Lin == t.ltot) {
    cid = t.leaf_cell[k];
    v = stock_leaf(t, p, cid, theta2);
  } else {
    cid = cell_at(Lin, k, t.ltot);
    v = load_node(t, cid);
  }
  int w = blockDim.x;   // nodes of the current level held by this block
  for (int L = Lin; L > Lout; L--) {
    if (tid < w) {
      put_node(sm, tid, v, cid);
      for (int q = 0; q < 5; q++) sq[q][tid] = v.q[q];
    }
    __syncthreads();
    w >>= 1;
    if (tid < w) {
      const StockNode a = get_node(sm, sq, 2 * tid), b = get_node(sm, sq, 2 * tid + 1);
      cid = sm.cid[2 * tid] - 1;   // the first child of c is c + 1
      v = stock_parent(t, cid, a, b, theta2);
    }
    __syncthreads();
  }
}

// ---- hmax update (KDTree::UpdateHmaxValues) --------------------------------------------
// hmax and hbox from the solved h (cdistsqd keeps its value), the same level scheme.
struct HmaxSmem {
  double d[7][kStockBlock];   // hbmin, hbmax, hmax
  int n[kStockBlock], cid[kStockBlock];
};

__global__ void __launch_bounds__(kStockBlock) k_update_hmax(Tree t, Particles p, int Lin, int Lout) {
  __shared__ HmaxSmem sm;
  const int tid = threadIdx.x;
  const int k = blockIdx.x * blockDim.x + tid;
  double hbmin[3], hbmax[3], hmax = 0.0;
  int cid, n;
  if (Lin == t.ltot) {
    cid = t.leaf_cell[k];
    const int first = t.cell_first[cid];
    n = t.cell_n[cid];
    for (int q = 0; q < 3; q++) { hbmin[q] = kBig; hbmax[q] = -kBig; }
    for (int j = 0; j < n; j++) {
      const int s = first + j;
      const double xs[3] = {p.x[s], p.y[s], p.z[s]};
      const double hh = p.h[s];
      hmax = kmax(hmax, hh);
      const double h2 = __dmul_rn(kKernRange, hh);
      for (int q = 0; q < 3; q++) {
        hbmin[q] = kmin(hbmin[q], __dsub_rn(xs[q], h2));
        hbmax[q] = kmax(hbmax[q], __dadd_rn(xs[q], h2));
      }
    }
    t.geom[cid].hmax = hmax;
    CellBox hb;
    for (int q = 0; q < 3; q++) { hb.bbmin[q] = hbmin[q]; hb.bbmax[q] = hbmax[q]; }
    t.hbox[cid] = hb;
  } else {
    cid = cell_at(Lin, k, t.ltot);
    n = t.cell_n[cid];
    const CellBox hb = t.hbox[cid];
    for (int q = 0; q < 3; q++) { hbmin[q] = hb.bbmin[q]; hbmax[q] = hb.bbmax[q]; }
    hmax = t.geom[cid].hmax;
  }
  int w = blockDim.x;
  for (int L = Lin; L > Lout; L--) {
    if (tid < w) {
      for (int q = 0; q < 3; q++) { sm.d[q][tid] = hbmin[q]; sm.d[3 + q][tid] = hbmax[q]; }
      sm.d[6][tid] = hmax;
      sm.n[tid] = n;
      sm.cid[tid] = cid;
    }
    __syncthreads();
    w >>= 1;
    if (tid < w) {
      hmax = 0.0;
      for (int q = 0; q < 3; q++) { hbmin[q] = kBig; hbmax[q] = -kBig; }
      for (int ch = 2 * tid; ch <= 2 * tid + 1; ch++) {
        if (sm.n[ch] <= 0) continue;
        hmax = kmax(hmax, sm.d[6][ch]);
        for (int q = 0; q < 3; q++) {
          hbmin[q] = kmin(sm.d[q][ch], hbmin[q]);
          hbmax[q] = kmax(sm.d[3 + q][ch], hbmax[q]);
        }
      }
      n = sm.n[2 * tid] + sm.n[2 * tid + 1];
      cid = sm.cid[2 * tid] - 1;
      t.geom[cid].hmax = hmax;
      CellBox hb;
      for (int q = 0; q < 3; q++) { hb.bbmin[q] = hbmin[q]; hb.bbmax[q] = hbmax[q]; }
      t.hbox[cid] = hb;
    }
    __syncthreads();
  }
}

// The level launches of a bottom-up pass: level ltot -> ... -> 0.
template <class F>
int for_stock_levels(int ltot, F&& launch) {
  int launches = 0;
  for (int Lin = ltot; Lin > 0;) {
    const int Lout = Lin > kStockLevels ? Lin - kStockLevels : 0;
    const int nodes = 1 << Lin;
    const int block = nodes < kStockBlock ? nodes : kStockBlock;
    launch(nodes / block, block, Lin, Lout);
    launches++;
    Lin = Lout;
  }
  if (ltot == 0) { launch(1, 1, 0, 0); launches++; }
  return launches;
}

int grid_for(int n, int block, int maxblocks = 152 * 16) {
  int g = (n + block - 1) / block;
  if (g < 1) g = 1;
  return g < maxblocks ? g : maxblocks;
}

}  // namespace

int sort_padded_size(int n) {
  int P = kSortBlock;
  while (P < n) P <<= 1;
  return P;
}

int partition_blocks(int n) { return (n + kScanBlock - 1) / kScanBlock; }

int radix_tiles(int n) { return (n + kRadixTile - 1) / kRadixTile; }

int launch_build_tree(const BuildArgs& a, cudaStream_t st) {
  int launches = 0;
  const int n = a.n;
  k_root_box_init<<<1, 32, 0, st>>>(a.rootkey);
  k_root_box<<<grid_for(n, 256, 152 * 4), 256, 0, st>>>(a.in.x, a.in.y, a.in.z, a.in.h, n, a.rootkey);
  k_root_box_store<<<1, 32, 0, st>>>(a.rootkey, a.ibox);
  launches += 3;
  k_sort_init<<<dim3(grid_for(n, 256), 3), 256, 0, st>>>(a.in.x, a.in.y, a.in.z, n, n, a.sort);
  launches += 1;
  {
    // radix passes ping-pong between the sort arrays and (key2, lists_b); eight passes
    // end in the sort arrays
    RadixArgs r{};
    r.n = n;
    r.ntiles = radix_tiles(n);
    r.hist = a.radix_hist;
    r.tot = a.radix_tot;
    const dim3 grid(r.ntiles, 3);
    // the staged tile (48 KB) is above the default dynamic shared-memory limit
    cudaFuncSetAttribute(k_radix_scatter, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) kRadixScatterSmem);
    constexpr int kPasses = (64 - kRadixSkipBits) / 8;   // an even count: ends in the sort arrays
    static_assert(kPasses % 2 == 0, "the radix passes must end in the sort arrays");
    for (int pass = 0; pass < kPasses; pass++) {
      for (int q = 0; q < 3; q++) {
        const bool even = (pass & 1) == 0;
        r.src_key[q] = even ? a.sort.key[q] : a.key2[q];
        r.src_idx[q] = even ? a.sort.idx[q] : a.lists_b[q];
        r.dst_key[q] = even ? a.key2[q] : a.sort.key[q];
        r.dst_idx[q] = even ? a.lists_b[q] : a.sort.idx[q];
      }
      const int shift = kRadixSkipBits + 8 * pass;
      k_radix_hist<<<grid, 256, 0, st>>>(r, shift);
      k_radix_scan<<<dim3(256, 3), 1024, 0, st>>>(r);
      k_radix_scatter<<<grid, 256, kRadixScatterSmem, st>>>(r, shift);
      launches += 3;
    }
    k_radix_fixup<<<dim3(grid_for(n, 256), 3), 256, 0, st>>>(a.sort, n);
    launches += 1;
  }
  BuildLists cur, nxt;
  for (int q = 0; q < 3; q++) { cur.l[q] = a.sort.idx[q]; nxt.l[q] = a.lists_b[q]; }
  const int nbl = (n + kPartTile - 1) / kPartTile;   // tiles of the level partition
  // levels from L0 on run in shared memory, one block per segment of level L0
  int L0 = 0;
  while (L0 < a.ltot && ((n + (1 << L0) - 1) >> L0) > kDeepMax) L0++;
  if (!a.deep_inv) L0 = a.ltot;
  for (int l = 0; l < L0; l++) {
    const int nseg = 1 << l;
    unsigned char* side = a.side[l & 1];
    k_split_prepare_next<<<(nseg + 127) / 128, 128, 0, st>>>(l, cur, a.in.x, a.in.y, a.in.z, a.heap_first,
                                                              a.heap_n, a.ibox, a.seg_axis, a.seg_axis_next);
    launches += 1;
    if (l == 0) {   // later levels get their marks from the previous level's partition
      k_mark_side<<<grid_for(n, 256), 256, 0, st>>>(l, n, cur, a.seg_axis, side);
      launches += 1;
    }
    k_part_level<<<3 * nbl, kPartThreads, 0, st>>>(l, n, cur, nxt, side,
                                                  l + 1 < L0 ? a.side[(l + 1) & 1] : nullptr, a.seg_axis_next,
                                                  a.heap_ones_before, nbl, a.part);
    launches += 1;
    BuildLists tmp = cur; cur = nxt; nxt = tmp;
  }
  if (L0 < a.ltot) {
    cudaFuncSetAttribute(k_build_deep, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) sizeof(DeepSmem));
    k_build_deep<<<1 << L0, kDeepThreads, sizeof(DeepSmem), st>>>(L0, a.ltot, cur, a.deep_inv, a.in.x, a.in.y, a.in.z,
                                                   a.heap_first, a.heap_n, a.ibox);
    launches++;
  }
  k_gather_leaf_order<<<grid_for(n, 256), 256, 0, st>>>(n, cur.l[0], a.in, a.p, a.id_out, a.slot_of);
  launches += 1;
  launches += for_stock_levels(a.tree.ltot, [&](int grid, int block, int Lin, int Lout) {
    k_stock<<<grid, block, 0, st>>>(a.tree, a.p, a.thetamaxsqd, Lin, Lout);
  });
  return launches;
}

int launch_update_hmax(const Tree& t, const Particles& p, cudaStream_t st) {
  return for_stock_levels(t.ltot, [&](int grid, int block, int Lin, int Lout) {
    k_update_hmax<<<grid, block, 0, st>>>(t, p, Lin, Lout);
  });
}

}  // namespace gsph

// ======================================================================================
// Allocation-free KD-tree ordering.
//
// For callers that cannot allocate device memory themselves — code whose device memory
// is owned by another allocator (a pool that has reserved the whole GPU), or a
// time-critical loop where cudaMalloc's implicit device synchronisation is not
// acceptable.  The scratch this computation needs lives in one file-scope device array
// of fixed size, held by every GPU that loads the library until the process exits.
// ======================================================================================
namespace gsph {
namespace {

constexpr int kNaMaxN = 32768;                              // particles
constexpr int kNaMaxLtot = 13;                              // tree levels
constexpr int kNaMaxCell = (1 << (kNaMaxLtot + 1)) - 1;     // depth-first cells
constexpr int kNaMaxNb = (kNaMaxN + kScanBlock - 1) / kScanBlock;

struct NoAllocScratch {
  unsigned long long key[3][kNaMaxN];
  int idx[3][kNaMaxN];
  int listb[3][kNaMaxN];
  double ibox[6 * kNaMaxCell];
  int heap_first[kNaMaxCell];
  int heap_n[kNaMaxCell];
  int heap_ones[kNaMaxCell];
  int blocksum[3 * kNaMaxNb];
  unsigned long long rootkey[8];
  unsigned char side[kNaMaxN];
  unsigned char seg_axis[(kNaMaxCell + 1) / 2];
};

static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

// Device address of g_noalloc_scratch and the SM count, looked up once per device (host
// code cannot use the symbol itself as a device pointer).  The cached address belongs to
// the context that was current at the lookup (the device's primary context); after a
// cudaDeviceReset, or with another context made current, it no longer names the array.
constexpr int kNaMaxDevices = 64;
NoAllocScratch* g_noalloc_ptr[kNaMaxDevices] = {};
int g_noalloc_sms[kNaMaxDevices] = {};

// Heap-indexed segment tables of level l (block l): first, count and the number of
// second-child positions before each segment.
__global__ void __launch_bounds__(1024) k_noalloc_heap_tables(int n, NoAllocScratch* s) {
  __shared__ int ws[33];
  const int l = blockIdx.x;
  const int nseg = 1 << l;
  int carry = 0;
  for (int base = 0; base < nseg; base += 1024) {
    const int q = base + threadIdx.x;
    int f = 0, c = n;
    if (q < nseg) {
      for (int lev = l - 1; lev >= 0; lev--) {
        const int half = c >> 1;
        if ((q >> lev) & 1) { f += half; c -= half; } else { c = half; }
      }
    }
    const int ones = q < nseg ? c - (c >> 1) : 0;
    int total;
    const int ex = block_exscan(ones, ws, total);
    if (q < nseg) {
      const int h = nseg - 1 + q;
      s->heap_first[h] = f;
      s->heap_n[h] = c;
      s->heap_ones[h] = carry + ex;
    }
    carry += total;
  }
}

}  // namespace
}  // namespace gsph

// Leaf-cell order of the reference KD-tree (KDTree::BuildTree, src/Tree/KDTree.cpp:219-595)
// computed without allocating: see include/gsph_gb300.h.
extern "C" int32_t gsph_kdtree_order_noalloc(const double* x, const double* y, const double* z,
                                             const double* h, int32_t n, int32_t nleafmax,
                                             int32_t* order, void* stream) {
  using namespace gsph;
  if (!x || !y || !z || !h || !order || n < 1 || nleafmax < 1) return -1;   // GSPH_ERR_INVALID
  int ltot = 0;
  while ((double) nleafmax * (double) (1 << ltot) < (double) n && ltot <= kNaMaxLtot) ltot++;
  if (n > kNaMaxN || ltot > kNaMaxLtot) return -6;                          // GSPH_ERR_CAPACITY
  // an error left pending by the caller's earlier work is reported, not taken as ours
  // (and not cleared: it stays for the caller to read)
  if (cudaPeekAtLastError() != cudaSuccess) return -2;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kNaMaxDevices) return -2;
  if (!g_noalloc_ptr[dev]) {
    NoAllocScratch* p = nullptr;
    if (cudaGetSymbolAddress((void**) &p, g_noalloc_scratch) != cudaSuccess || !p) return -2;
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1) return -2;
    g_noalloc_sms[dev] = sms;
    g_noalloc_ptr[dev] = p;
  }
  NoAllocScratch* s = g_noalloc_ptr[dev];
  const int sms = g_noalloc_sms[dev];
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  k_noalloc_heap_tables<<<ltot + 1, 1024, 0, st>>>(n, s);
  if (cudaGetLastError() != cudaSuccess) return -2;   // a bad stream fails here, before more work
  k_root_box_init<<<1, 32, 0, st>>>(s->rootkey);
  k_root_box<<<grid_for(n, 256, sms * 4), 256, 0, st>>>(x, y, z, h, n, s->rootkey);
  k_root_box_store<<<1, 32, 0, st>>>(s->rootkey, s->ibox);
  SortArrays sa;
  for (int q = 0; q < 3; q++) { sa.key[q] = s->key[q]; sa.idx[q] = s->idx[q]; }
  const int P = sort_padded_size(n);
  k_sort_init<<<dim3(grid_for(P, 256), 3), 256, 0, st>>>(x, y, z, n, P, sa);
  k_bitonic_smem<<<dim3(P / kSortBlock, 3), kSortBlock / 2, 0, st>>>(sa, 2, kSortBlock, kSortBlock / 2);
  for (int k = 2 * kSortBlock; k <= P; k <<= 1) {
    for (int j = k >> 1; j >= kSortBlock; j >>= 1)
      k_bitonic_global<<<dim3(grid_for(P / 2, 256, 1 << 20), 3), 256, 0, st>>>(sa, P, k, j);
    k_bitonic_smem<<<dim3(P / kSortBlock, 3), kSortBlock / 2, 0, st>>>(sa, k, k, kSortBlock / 2);
  }
  BuildLists cur, nxt;
  for (int q = 0; q < 3; q++) { cur.l[q] = s->idx[q]; nxt.l[q] = s->listb[q]; }
  const int nb = partition_blocks(n);
  for (int l = 0; l < ltot; l++) {
    const int nseg = 1 << l;
    k_split_prepare<<<(nseg + 127) / 128, 128, 0, st>>>(l, cur, x, y, z, s->heap_first, s->heap_n, s->ibox,
                                                         s->seg_axis);
    k_mark_side<<<grid_for(n, 256), 256, 0, st>>>(l, n, cur, s->seg_axis, s->side);
    k_part_count<<<dim3(nb, 3), 1024, 0, st>>>(n, cur, s->side, s->blocksum, nb);
    k_part_scan<<<dim3(1, 3), 1024, 0, st>>>(s->blocksum, nb);
    k_part_scatter<<<dim3(nb, 3), 1024, 0, st>>>(l, n, cur, nxt, s->side, s->blocksum, nb, s->heap_ones);
    BuildLists tmp = cur; cur = nxt; nxt = tmp;
  }
  if (cudaMemcpyAsync(order, cur.l[0], sizeof(int) * (size_t) n, cudaMemcpyDeviceToDevice, st) != cudaSuccess)
    return -2;
  return cudaGetLastError() == cudaSuccess ? 0 : -2;
}
