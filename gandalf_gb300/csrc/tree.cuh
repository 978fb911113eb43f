// Host-side launchers of the tree kernels (tree.cu).
#pragma once
#include "gsph_state.cuh"

namespace gsph {

struct SortArrays {
  unsigned long long* key[3];   // order-preserving coordinate keys, padded length P
  int* idx[3];                  // particle indices, padded length P
};

// One radix-sort pass over the three axes' (key, index) lists.
struct RadixArgs {
  int n, ntiles;
  const unsigned long long* src_key[3];
  const int* src_idx[3];
  unsigned long long* dst_key[3];
  int* dst_idx[3];
  int* hist;                    // 3 x 256 x ntiles, digit-major
  int* tot;                     // 3 x 256
};

struct BuildLists {
  int* l[3];                    // per-axis position lists of particle indices
};

// Cross-block state of the single-pass level partition (tree.cu k_part_level).
struct PartitionState {
  unsigned long long* tiles;    // 3 * partition_blocks(n) tile words
  unsigned* ticket;             // next tile ticket (0 between launches)
  unsigned* epoch;              // launch epoch of the tile words
  unsigned* status;             // kStatusPartitionWait when a look-back wait gave up
};

struct InputArrays {            // input order, fp64
  const double *x, *y, *z, *vx, *vy, *vz, *m, *u, *h;
};

struct BuildArgs {
  int n, ltot, P;
  InputArrays in;
  SortArrays sort;
  int* lists_b[3];              // second buffer of the ping-pong position lists (length n)
  unsigned long long* key2[3];  // second key buffer of the radix sort (length n)
  int* radix_hist;              // 3 x 256 x radix_tiles(n)
  int* radix_tot;               // 3 x 256
  int* deep_inv;                // n: global -> local id of the shared-memory deep levels
  unsigned char* side[2];       // per particle: 0 first child, 1 second child (this level, next level)
  unsigned char* seg_axis;      // per segment of the current level
  unsigned char* seg_axis_next; // per segment of the next level
  PartitionState part;
  unsigned long long* rootkey;  // 6
  double* ibox;                 // inherited boxes, heap-indexed, 6 per cell
  const int* heap_first;        // heap-indexed segment tables (static per N)
  const int* heap_n;
  const int* heap_ones_before;
  Particles p;                  // leaf-ordered destination
  int* id_out;                  // input index of each slot
  int* slot_of;                 // slot of each input index (the inverse permutation)
  Tree tree;
  double thetamaxsqd;
};

int sort_padded_size(int n);
int partition_blocks(int n);
int radix_tiles(int n);
int launch_build_tree(const BuildArgs& a, cudaStream_t st);   // returns kernels launched
int launch_update_hmax(const Tree& t, const Particles& p, cudaStream_t st);   // returns kernels launched

}  // namespace gsph
