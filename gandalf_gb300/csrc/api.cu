// C ABI of the GB300 grad-h SPH + KD-tree gravity step (declared in include/gsph_gb300.h).
//
// Host orchestration of one step, following HydroTree/GradhSphTree
// (src/Tree/HydroTree.cpp:309-441, src/GradhSph/GradhSphTree.cpp:82-657):
//   build tree -> h-rho solve -> hmax update -> hydro or hydro + gravity forces.
// Device memory is owned by the context and sized for the largest N seen.  Every launch
// goes to the context's stream; a step synchronises once at its end to read the
// kernels' status word.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/gsph_gb300.h"
#include "gsph_state.cuh"
#include "kernels.cuh"
#include "batch.cuh"
#include "integrate.cuh"
#include "mixed_state.cuh"
#include "stars.cuh"
#include "tree.cuh"

using namespace gsph;

namespace {

thread_local int g_create_error = GSPH_OK;

struct Buf {
  void* p = nullptr;
  size_t bytes = 0;
};

}  // namespace

struct gsph_ctx {
  gsph_config cfg;
  int device = 0;
  cudaStream_t stream = nullptr;      // stream all work is launched on
  cudaStream_t own_stream = nullptr;  // the context's own stream
  unsigned launches = 0;              // kernels launched since the step began
  std::string err;
  std::vector<Buf> bufs;     // everything allocated for the current capacity
  int cap = 0;               // particle capacity of the allocations
  int cap_ncell = 0;
  int n = 0;                 // particles of the current set
  bool have_particles = false, have_tree = false, have_props = false, have_forces = false;
  // topology of the current n
  int ltot = 0, ncell = 0, nleaf = 0, P = 0, lpg = 4;
  // device arrays
  double* in[9] = {};        // x y z vx vy vz m u h (input order)
  double* f[30] = {};        // leaf-order fields (see kF* below)
  int* id = nullptr;
  int *cell_first = nullptr, *cell_n = nullptr, *cell_parent = nullptr, *leaf_cell = nullptr;
  unsigned char* cell_level = nullptr;
  int *heap_first = nullptr, *heap_n = nullptr, *heap_ones = nullptr;
  CellGeom* geom = nullptr;
  CellBox *bb = nullptr, *hbox = nullptr;
  CellMoment* mom = nullptr;
  unsigned long long* key[3] = {};
  int* idx[3] = {};
  int* listb[3] = {};
  unsigned long long* key2[3] = {};
  int* deep_inv = nullptr;
  int* slot_of = nullptr;                 // slot of each input particle (inverse of id)
  int* dens_next = nullptr;               // FP64 h solve: leaf counter of its persistent warps
  double2* dens_comp = nullptr;           // FP64 h solve: per-warp compact lists
  int *radix_hist = nullptr, *radix_tot = nullptr;
  unsigned char *side = nullptr, *side2 = nullptr, *seg_axis = nullptr, *seg_axis_next = nullptr;
  unsigned long long* part_tiles = nullptr;
  unsigned* part_sync = nullptr;   // ticket, epoch
  unsigned long long* rootkey = nullptr;
  double* ibox = nullptr;
  unsigned long long* counters = nullptr;    // [0] status, [1..5] counts
  double* scratch_out = nullptr;             // n doubles for field scatter
  // array-of-structures import / export
  void* aos = nullptr;                 // device copy of records that are not page-locked
  size_t aos_bytes = 0;
  int64_t aos_stride = 0;
  bool bactive = false;                // records carry flags: block-timestep semantics
  double* aos_out = nullptr;           // staged write-back: fields x n, input order
  size_t aos_out_bytes = 0;
  // recording
  int record = 0, rec_max = 0;
  int* rec_sph_cnt = nullptr;
  int* rec_sph_ids = nullptr;
  unsigned long long *rec_dir_cnt = nullptr, *rec_dir_hash = nullptr, *rec_cell_cnt = nullptr,
                     *rec_cell_hash = nullptr;
  size_t rec_bytes = 0;
  // full direct-sum and multipole-cell lists (gsph_set_list_recording)
  int rec_dir_max = 0, rec_cell_max = 0;
  int *rec_dir_n = nullptr, *rec_dir_ids = nullptr, *rec_cell_n = nullptr, *rec_cell_ids = nullptr;
  size_t rec_full_bytes = 0;
  // mixed-precision mirrors and the heavy-leaf hand-over list
  float4 *mp_pos_hi = nullptr, *mp_pos_lo = nullptr, *mp_vel = nullptr, *mp_hyd = nullptr, *mp_aux = nullptr;
  float4 *mc_geo_hi = nullptr, *mc_geo_lo = nullptr, *mc_com_hi = nullptr, *mc_com_lo = nullptr, *mc_quad = nullptr,
         *mc_bbmin = nullptr, *mc_bbmax = nullptr, *mc_hbmin = nullptr, *mc_hbmax = nullptr;
  float4* mc_meta = nullptr;
  int* heavy_leaves = nullptr;
  int* heavy_count = nullptr;   // [0] current heavy count, [1] wide-tier count, [2] [3] snapshots
  int* wide_leaves = nullptr;   // leaves of the mixed h solve's wide tier
  int max_leaf = 8;
  // star particles: 8 input arrays (x y z vx vy vz m h) then 7 results (a, adot, gpot)
  int nstar = 0, star_cap = 0;
  double* star_buf = nullptr;
  float4* star_f = nullptr;               // mixed form: 2 x star_cap (hi xyz m, lo xyz h)
  std::vector<float4> star_f_host;        // staging of the last upload
  bool have_star_forces = false;
  // KDK integration with block timesteps (gsph_kdk_*)
  bool kdk = false;
  bool keep_current = false;          // results live in the KDK state (input order), complete
  KdkParams kp{};
  KdkGlobal* kg = nullptr;
  double* kdk_buf = nullptr;          // r0 v0 a0 (9), u0 dudt0 dt dt_next tlast (5), keep (17): x cap
  int* kdk_ibuf = nullptr;            // nlast nstep level levelneib bt_list: x cap
  unsigned char* kdk_flags = nullptr;
  unsigned char* leaf_active = nullptr;
  int *leaf_level = nullptr, *leaf_lvn = nullptr;
  int kdk_cap = 0;
  cudaGraph_t kdk_graph = nullptr;
  cudaGraphExec_t kdk_exec = nullptr;
  int kdk_graph_steps = 0;
  unsigned kdk_graph_launches = 0;
  // phase timing of gsph_kdk_steps: begin/end event pairs around each tree build, h solve
  // and force pass (graph nodes when the steps are captured)
  std::vector<cudaEvent_t> pev;
  std::vector<int> pkind;
  size_t pused = 0;
  bool ptiming = false;
  // CheckTimesteps repeat passes: captured as conditional graph nodes, nested two deep
  cudaStream_t cond_stream[2] = {};
  cudaStream_t cond_saved[2] = {};
  int in_body = 0;                       // > 0 while capturing a conditional body
  unsigned long long* kdk_snap = nullptr;   // first-pass counter snapshots, 8 per step
  int kdk_snap_steps = 0;
  unsigned kdk_cond_launches = 0;        // kernels of one repeat pass
  gsph_kdk_timing kdk_timing{};          // of the last gsph_kdk_steps
  // CUDA graph of the whole step (gsph_step_graph), valid for one capture key
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t graph_exec = nullptr;
  bool graph_valid = false;
  bool capturing = false;
  unsigned graph_launches = 0;
  // tuned list depths of the mixed kernels (0: compiled maxima)
  int near_depth = 0, cell_depth = 0, gather_depth = 0;
  // timing
  cudaEvent_t ev[5] = {};
  gsph_stats last{};
};

namespace {

enum {
  kFX = 0, kFY, kFZ, kFVX, kFVY, kFVZ, kFM, kFU, kFH, kFH0, kFRho, kFInvOmega, kFZeta, kFHfactor,
  kFHrangesqd, kFPressure, kFSound, kFAX, kFAY, kFAZ, kFAGX, kFAGY, kFAGZ, kFGpot, kFDudt, kFDivV,
  kFGpotHydro, kFInvH, kFInvRho, kFFac, kNumFields
};
static_assert(kNumFields == 30, "gsph_ctx::f holds kNumFields pointers");

int fail(gsph_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  return code;
}

int cuda_fail(gsph_ctx* c, cudaError_t e, const char* where) {
  return fail(c, GSPH_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

#define GSPH_CUDA(call)                                   \
  do {                                                    \
    cudaError_t e_ = (call);                              \
    if (e_ != cudaSuccess) return cuda_fail(c, e_, #call); \
  } while (0)

void free_all(gsph_ctx* c) {
  for (Buf& b : c->bufs) if (b.p) cudaFree(b.p);
  c->bufs.clear();
  c->cap = 0;
  c->cap_ncell = 0;
}

void kdk_free(gsph_ctx* c);
KdkState make_kdk_state(gsph_ctx* c);
KdkLeaf make_kdk_leaf(gsph_ctx* c);
int ensure_kdk_buffers(gsph_ctx* c);
const double* kdk_field_source(gsph_ctx* c, int leaf_field);

void drop_graph(gsph_ctx* c) {
  if (c->graph_exec) cudaGraphExecDestroy(c->graph_exec);
  if (c->graph) cudaGraphDestroy(c->graph);
  c->graph_exec = nullptr;
  c->graph = nullptr;
  c->graph_valid = false;
}

// The K-step KDK graph: kept across gsph_kdk_setup calls while the buffers, the tree shape,
// the recording setting and the KDK parameters it captured stay the same.
void drop_kdk_graph(gsph_ctx* c) {
  if (c->kdk_exec) cudaGraphExecDestroy(c->kdk_exec);
  if (c->kdk_graph) cudaGraphDestroy(c->kdk_graph);
  c->kdk_exec = nullptr;
  c->kdk_graph = nullptr;
  c->kdk_graph_steps = 0;
}

template <class T>
int alloc(gsph_ctx* c, T*& ptr, size_t count) {
  void* p = nullptr;
  const size_t bytes = std::max<size_t>(count, 1) * sizeof(T);
  cudaError_t e = cudaMalloc(&p, bytes);
  if (e != cudaSuccess) return cuda_fail(c, e, "cudaMalloc");
  c->bufs.push_back({p, bytes});
  ptr = static_cast<T*>(p);
  return GSPH_OK;
}

int tree_levels(int n, int nleafmax) {
  int l = 0;
  while ((double) nleafmax * std::pow(2.0, l) < (double) n) l++;
  return l;
}

// Host tables of the tree shape for n particles (KDTree::CreateTreeStructure layout).
struct Shape {
  std::vector<int> cell_first, cell_n, cell_parent, leaf_cell, heap_first, heap_n, heap_ones;
  std::vector<unsigned char> cell_level;
};

void make_shape(int n, int ltot, Shape& s) {
  const int ncell = 2 * (1 << ltot) - 1;
  s.cell_first.assign(ncell, 0); s.cell_n.assign(ncell, 0); s.cell_parent.assign(ncell, -1);
  s.cell_level.assign(ncell, 0); s.leaf_cell.assign(1 << ltot, 0);
  s.heap_first.assign(ncell, 0); s.heap_n.assign(ncell, 0); s.heap_ones.assign(ncell, 0);
  struct Item { int c, h, level, first, cnt, parent; };
  std::vector<Item> st;
  st.push_back({0, 0, 0, 0, n, -1});
  while (!st.empty()) {
    Item it = st.back();
    st.pop_back();
    s.cell_first[it.c] = it.first; s.cell_n[it.c] = it.cnt; s.cell_parent[it.c] = it.parent;
    s.cell_level[it.c] = (unsigned char) it.level;
    s.heap_first[it.h] = it.first; s.heap_n[it.h] = it.cnt;
    if (it.level == ltot) {
      s.leaf_cell[it.h - ((1 << ltot) - 1)] = it.c;
      continue;
    }
    const int half = it.cnt / 2;
    const int c2 = it.c + (1 << (ltot - it.level));
    st.push_back({c2, 2 * it.h + 2, it.level + 1, it.first + half, it.cnt - half, it.c});
    st.push_back({it.c + 1, 2 * it.h + 1, it.level + 1, it.first, half, it.c});
  }
  for (int l = 0; l <= ltot; l++) {
    int acc = 0;
    for (int q = 0; q < (1 << l); q++) {
      const int h = (1 << l) - 1 + q;
      s.heap_ones[h] = acc;
      acc += s.heap_n[h] - s.heap_n[h] / 2;
    }
  }
}

int ensure_capacity(gsph_ctx* c, int n) {
  const int ltot = tree_levels(n, c->cfg.nleafmax);
  if (ltot > 23) return fail(c, GSPH_ERR_UNSUPPORTED, "tree deeper than 23 levels");
  if (c->cfg.precision == GSPH_PRECISION_MIXED && n > mixed_max_particles())
    return fail(c, GSPH_ERR_UNSUPPORTED, "the mixed form takes at most 2^27 particles");
  const int ncell = 2 * (1 << ltot) - 1;
  const int P = sort_padded_size(n);
  bool fresh = false;
  if (n > c->cap || ncell > c->cap_ncell || P > sort_padded_size(std::max(c->cap, 1))) {
    fresh = true;
    free_all(c);
    const int capn = n, capc = ncell, capP = P;
    int rc = GSPH_OK;
    for (int q = 0; q < 9 && rc == GSPH_OK; q++) rc = alloc(c, c->in[q], capn);
    for (int q = 0; q < kNumFields && rc == GSPH_OK; q++) rc = alloc(c, c->f[q], capn);
    if (rc == GSPH_OK) rc = alloc(c, c->id, capn);
    if (rc == GSPH_OK) rc = alloc(c, c->cell_first, capc);
    if (rc == GSPH_OK) rc = alloc(c, c->cell_n, capc);
    if (rc == GSPH_OK) rc = alloc(c, c->cell_parent, capc);
    if (rc == GSPH_OK) rc = alloc(c, c->cell_level, capc);
    if (rc == GSPH_OK) rc = alloc(c, c->leaf_cell, (capc + 1) / 2);
    if (rc == GSPH_OK) rc = alloc(c, c->heap_first, capc);
    if (rc == GSPH_OK) rc = alloc(c, c->heap_n, capc);
    if (rc == GSPH_OK) rc = alloc(c, c->heap_ones, capc);
    if (rc == GSPH_OK) rc = alloc(c, c->geom, capc);
    if (rc == GSPH_OK) rc = alloc(c, c->bb, capc);
    if (rc == GSPH_OK) rc = alloc(c, c->hbox, capc);
    if (rc == GSPH_OK) rc = alloc(c, c->mom, capc);
    for (int q = 0; q < 3 && rc == GSPH_OK; q++) rc = alloc(c, c->key[q], capP);
    for (int q = 0; q < 3 && rc == GSPH_OK; q++) rc = alloc(c, c->idx[q], capP);
    for (int q = 0; q < 3 && rc == GSPH_OK; q++) rc = alloc(c, c->listb[q], capn);
    for (int q = 0; q < 3 && rc == GSPH_OK; q++) rc = alloc(c, c->key2[q], capn);
    if (rc == GSPH_OK) rc = alloc(c, c->radix_hist, (size_t) 3 * 256 * radix_tiles(capn));
    if (rc == GSPH_OK) rc = alloc(c, c->radix_tot, 3 * 256);
    if (rc == GSPH_OK) rc = alloc(c, c->deep_inv, capn);
    if (rc == GSPH_OK) rc = alloc(c, c->slot_of, capn);
    if (rc == GSPH_OK) rc = alloc(c, c->dens_next, 1);
    if (rc == GSPH_OK && c->cfg.precision != GSPH_PRECISION_MIXED) rc = alloc(c, c->dens_comp, density_fp64_scratch_entries());
    if (rc == GSPH_OK) rc = alloc(c, c->side, capn);
    if (rc == GSPH_OK) rc = alloc(c, c->side2, capn);
    if (rc == GSPH_OK) rc = alloc(c, c->seg_axis, (capc + 1) / 2);
    if (rc == GSPH_OK) rc = alloc(c, c->seg_axis_next, (capc + 1) / 2);
    if (rc == GSPH_OK) rc = alloc(c, c->part_tiles, 3 * (size_t) partition_blocks(capn));
    if (rc == GSPH_OK) rc = alloc(c, c->part_sync, 2);
    // the partition's tile words start invalid (flag 0) and its ticket counter at 0
    if (rc == GSPH_OK && cudaMemset(c->part_tiles, 0, sizeof(unsigned long long) * 3 * (size_t) partition_blocks(capn)) != cudaSuccess)
      rc = fail(c, GSPH_ERR_CUDA, "cudaMemset");
    if (rc == GSPH_OK && cudaMemset(c->part_sync, 0, 2 * sizeof(unsigned)) != cudaSuccess)
      rc = fail(c, GSPH_ERR_CUDA, "cudaMemset");
    if (rc == GSPH_OK) rc = alloc(c, c->rootkey, 8);
    if (rc == GSPH_OK) rc = alloc(c, c->ibox, 6 * ((size_t) 2 * capc + 3));
    if (rc == GSPH_OK) rc = alloc(c, c->counters, 16);
    if (rc == GSPH_OK) rc = alloc(c, c->scratch_out, capn);
    if (c->cfg.precision == GSPH_PRECISION_MIXED) {
      float4** pf[5] = {&c->mp_pos_hi, &c->mp_pos_lo, &c->mp_vel, &c->mp_hyd, &c->mp_aux};
      for (int q = 0; q < 5 && rc == GSPH_OK; q++) rc = alloc(c, *pf[q], capn);
      float4** cf[9] = {&c->mc_geo_hi, &c->mc_geo_lo, &c->mc_com_hi, &c->mc_com_lo, &c->mc_quad,
                        &c->mc_bbmin, &c->mc_bbmax, &c->mc_hbmin, &c->mc_hbmax};
      for (int q = 0; q < 9 && rc == GSPH_OK; q++) rc = alloc(c, *cf[q], capc);
      if (rc == GSPH_OK) rc = alloc(c, c->mc_meta, capc);
    }
    if (rc == GSPH_OK) rc = alloc(c, c->heavy_leaves, (capc + 1) / 2);
    if (rc == GSPH_OK) rc = alloc(c, c->wide_leaves, (capc + 1) / 2);
    if (rc == GSPH_OK) rc = alloc(c, c->heavy_count, 4);
    if (rc != GSPH_OK) { free_all(c); return rc; }
    c->cap = capn;
    c->cap_ncell = capc;
    c->rec_bytes = 0;   // recording buffers were freed with the rest
    c->rec_full_bytes = 0;
    c->rec_dir_n = c->rec_dir_ids = c->rec_cell_n = c->rec_cell_ids = nullptr;
    c->rec_sph_cnt = nullptr;
  }
  if (fresh || n != c->n || ltot != c->ltot) { drop_graph(c); drop_kdk_graph(c); }
  if (fresh || n != c->n) c->kdk = false;   // a new particle set restarts any integration
  if (fresh || n != c->n || ltot != c->ltot || !c->have_particles) {
    Shape s;
    make_shape(n, ltot, s);
    cudaStream_t st = c->stream;
    GSPH_CUDA(cudaMemcpyAsync(c->cell_first, s.cell_first.data(), sizeof(int) * ncell, cudaMemcpyHostToDevice, st));
    GSPH_CUDA(cudaMemcpyAsync(c->cell_n, s.cell_n.data(), sizeof(int) * ncell, cudaMemcpyHostToDevice, st));
    GSPH_CUDA(cudaMemcpyAsync(c->cell_parent, s.cell_parent.data(), sizeof(int) * ncell, cudaMemcpyHostToDevice, st));
    GSPH_CUDA(cudaMemcpyAsync(c->cell_level, s.cell_level.data(), ncell, cudaMemcpyHostToDevice, st));
    GSPH_CUDA(cudaMemcpyAsync(c->leaf_cell, s.leaf_cell.data(), sizeof(int) * (1 << ltot), cudaMemcpyHostToDevice, st));
    GSPH_CUDA(cudaMemcpyAsync(c->heap_first, s.heap_first.data(), sizeof(int) * ncell, cudaMemcpyHostToDevice, st));
    GSPH_CUDA(cudaMemcpyAsync(c->heap_n, s.heap_n.data(), sizeof(int) * ncell, cudaMemcpyHostToDevice, st));
    GSPH_CUDA(cudaMemcpyAsync(c->heap_ones, s.heap_ones.data(), sizeof(int) * ncell, cudaMemcpyHostToDevice, st));
    GSPH_CUDA(cudaStreamSynchronize(st));   // host tables go out of scope
    int maxleaf = 0;
    for (int q = 0; q < (1 << ltot); q++) maxleaf = std::max(maxleaf, s.cell_n[s.leaf_cell[q]]);
    int p2 = 1;
    while (p2 < maxleaf) p2 <<= 1;
    if (p2 > 32) return fail(c, GSPH_ERR_UNSUPPORTED, "leaf cells hold more than 32 particles");
    c->lpg = 32 / p2;
    c->max_leaf = maxleaf;
  }
  c->n = n;
  c->ltot = ltot;
  c->ncell = ncell;
  c->nleaf = 1 << ltot;
  c->P = P;
  return GSPH_OK;
}

StarSet make_stars(const gsph_ctx* c) {
  StarSet s{};
  s.n = c->nstar;
  if (!c->nstar) return s;
  const double* b = c->star_buf;
  const size_t k = (size_t) c->star_cap;
  s.x = b; s.y = b + k; s.z = b + 2 * k; s.vx = b + 3 * k; s.vy = b + 4 * k; s.vz = b + 5 * k;
  s.m = b + 6 * k; s.h = b + 7 * k;
  double* o = c->star_buf + 8 * k;
  s.ax = o; s.ay = o + k; s.az = o + 2 * k; s.adotx = o + 3 * k; s.adoty = o + 4 * k; s.adotz = o + 5 * k;
  s.gpot = o + 6 * k;
  s.fhi = c->star_f;
  s.flo = c->star_f + k;
  return s;
}

SphParams make_params(const gsph_ctx* c) {
  SphParams p{};
  const gsph_config& cfg = c->cfg;
  p.stars = make_stars(c);
  p.h_fac = cfg.h_fac; p.h_converge = cfg.h_converge; p.alpha_visc = cfg.alpha_visc;
  p.beta_visc = cfg.beta_visc; p.gamma_eos = cfg.gamma_eos; p.temp0 = cfg.temp0; p.mu_bar = cfg.mu_bar;
  p.thetamaxsqd = cfg.thetamaxsqd;
  p.u_iso = cfg.temp0 / (cfg.gamma_eos - 1.0) / cfg.mu_bar;
  for (int k = 0; k < 3; k++) {
    p.boxmin[k] = cfg.boxmin[k]; p.boxmax[k] = cfg.boxmax[k];
    p.boxsize[k] = cfg.boxmax[k] - cfg.boxmin[k];
    p.boxhalf[k] = 0.5 * p.boxsize[k];
  }
  p.eos = cfg.eos; p.periodic = cfg.periodic; p.multipole = cfg.multipole; p.self_gravity = cfg.self_gravity;
  p.compensated = cfg.precision == GSPH_PRECISION_MIXED && cfg.compensated ? 1 : 0;
  p.near_depth = c->near_depth; p.cell_depth = c->cell_depth; p.gather_depth = c->gather_depth;
  p.alpha_visc_f = (float) cfg.alpha_visc;
  p.ab_visc_f = (float) (cfg.beta_visc * cfg.alpha_visc);
  p.gm1_f = (float) (cfg.gamma_eos - 1.0);
  return p;
}

Particles make_particles(gsph_ctx* c) {
  Particles p{};
  p.n = c->n;
  p.id = c->id;
  double** f = c->f;
  p.x = f[kFX]; p.y = f[kFY]; p.z = f[kFZ]; p.vx = f[kFVX]; p.vy = f[kFVY]; p.vz = f[kFVZ];
  p.m = f[kFM]; p.u = f[kFU]; p.h = f[kFH]; p.h0 = f[kFH0];
  p.rho = f[kFRho]; p.invomega = f[kFInvOmega]; p.zeta = f[kFZeta]; p.hfactor = f[kFHfactor];
  p.hrangesqd = f[kFHrangesqd]; p.pressure = f[kFPressure]; p.sound = f[kFSound];
  p.ax = f[kFAX]; p.ay = f[kFAY]; p.az = f[kFAZ]; p.agx = f[kFAGX]; p.agy = f[kFAGY]; p.agz = f[kFAGZ];
  p.gpot = f[kFGpot]; p.dudt = f[kFDudt]; p.div_v = f[kFDivV]; p.gpot_hydro = f[kFGpotHydro];
  p.invh_p = f[kFInvH]; p.invrho_p = f[kFInvRho]; p.fac_p = f[kFFac];
  if (c->kdk || c->bactive) { p.active = c->leaf_active; p.level = c->leaf_level; p.lvn = c->leaf_lvn; }
  return p;
}

Tree make_tree(gsph_ctx* c) {
  Tree t{};
  t.n = c->n; t.ltot = c->ltot; t.ncell = c->ncell; t.nleaf = c->nleaf;
  t.cell_first = c->cell_first; t.cell_n = c->cell_n; t.cell_level = c->cell_level;
  t.cell_parent = c->cell_parent; t.leaf_cell = c->leaf_cell;
  t.geom = c->geom; t.bb = c->bb; t.hbox = c->hbox; t.mom = c->mom;
  return t;
}

MixedParticles make_mixed_particles(gsph_ctx* c) {
  return MixedParticles{c->mp_pos_hi, c->mp_pos_lo, c->mp_vel, c->mp_hyd, c->mp_aux};
}

MixedCells make_mixed_cells(gsph_ctx* c) {
  return MixedCells{c->mc_geo_hi, c->mc_geo_lo, c->mc_meta, c->mc_com_hi, c->mc_com_lo, c->mc_quad,
                    c->mc_bbmin, c->mc_bbmax, c->mc_hbmin, c->mc_hbmax};
}

bool mixed(const gsph_ctx* c) { return c->cfg.precision == GSPH_PRECISION_MIXED; }

DeviceCounters make_counters(gsph_ctx* c) {
  DeviceCounters d{};
  d.status = reinterpret_cast<unsigned*>(c->counters);
  d.density_pairs = c->counters + 1;
  d.hydro_pairs = c->counters + 2;
  d.direct_pairs = c->counters + 3;
  d.cell_pairs = c->counters + 4;
  d.exact_checks = c->counters + 5;
  d.record = c->record && c->rec_sph_cnt != nullptr;
  d.rec_max = c->rec_max;
  d.rec_sph_cnt = c->rec_sph_cnt; d.rec_sph_ids = c->rec_sph_ids;
  d.rec_dir_cnt = c->rec_dir_cnt; d.rec_dir_hash = c->rec_dir_hash;
  d.rec_cell_cnt = c->rec_cell_cnt; d.rec_cell_hash = c->rec_cell_hash;
  if (d.record && c->rec_dir_max > 0 && c->rec_dir_n) {
    d.rec_dir_max = c->rec_dir_max; d.rec_cell_max = c->rec_cell_max;
    d.rec_dir_n = c->rec_dir_n; d.rec_dir_ids = c->rec_dir_ids;
    d.rec_cell_n = c->rec_cell_n; d.rec_cell_ids = c->rec_cell_ids;
  }
  return d;
}

int check_config(const gsph_config* cfg, std::string& why) {
  if (!cfg) { why = "config is NULL"; return GSPH_ERR_INVALID; }
  if (cfg->ndim != 3) { why = "only ndim = 3 is implemented"; return GSPH_ERR_UNSUPPORTED; }
  if (cfg->nleafmax < 1 || cfg->nleafmax > 32) { why = "Nleafmax must be 1..32"; return GSPH_ERR_INVALID; }
  if (cfg->eos != GSPH_EOS_ENERGY_EQN && cfg->eos != GSPH_EOS_ISOTHERMAL) { why = "unknown gas_eos"; return GSPH_ERR_UNSUPPORTED; }
  if (cfg->multipole != GSPH_MONOPOLE && cfg->multipole != GSPH_QUADRUPOLE) { why = "unknown multipole"; return GSPH_ERR_UNSUPPORTED; }
  if (cfg->precision != GSPH_PRECISION_FP64 && cfg->precision != GSPH_PRECISION_MIXED) { why = "unknown precision"; return GSPH_ERR_INVALID; }
  if (cfg->self_gravity && cfg->periodic) { why = "periodic self-gravity needs Ewald sums (not implemented)"; return GSPH_ERR_UNSUPPORTED; }
  if ((cfg->compensated != 0 && cfg->compensated != 1) || cfg->reserved != 0) { why = "compensated must be 0 or 1"; return GSPH_ERR_INVALID; }
  if (!cfg->hydro_forces) { why = "hydro_forces = 0 is not implemented"; return GSPH_ERR_UNSUPPORTED; }
  if (!(cfg->h_fac > 0.0) || !(cfg->h_converge > 0.0) || !(cfg->gamma_eos > 1.0) || !(cfg->thetamaxsqd > 0.0)) {
    why = "h_fac, h_converge, thetamaxsqd must be > 0 and gamma_eos > 1"; return GSPH_ERR_INVALID;
  }
  if (cfg->periodic)
    for (int k = 0; k < 3; k++)
      if (!(cfg->boxmax[k] > cfg->boxmin[k])) { why = "periodic box has non-positive size"; return GSPH_ERR_INVALID; }
  return GSPH_OK;
}

int validate_host(gsph_ctx* c, int64_t n, const double* const* a) {
  for (int q = 0; q < 9; q++) if (!a[q]) return fail(c, GSPH_ERR_INVALID, "particle array is NULL");
  for (int64_t i = 0; i < n; i++) {
    for (int q = 0; q < 9; q++)
      if (!std::isfinite(a[q][i])) return fail(c, GSPH_ERR_INVALID, "non-finite particle data");
    if (!(a[6][i] > 0.0)) return fail(c, GSPH_ERR_INVALID, "particle mass must be > 0");
    if (!(a[8][i] > 0.0)) return fail(c, GSPH_ERR_INVALID, "smoothing length must be > 0");
    if (c->cfg.periodic)
      for (int k = 0; k < 3; k++)
        if (a[k][i] < c->cfg.boxmin[k] || a[k][i] >= c->cfg.boxmax[k])
          return fail(c, GSPH_ERR_INVALID, "particle outside the periodic box");
  }
  return GSPH_OK;
}

struct OutPtrs { double* p[9]; };

// A record field read as a double / int32 (offset -1: absent, the default).
__device__ __forceinline__ double rec_d(const unsigned char* r, int64_t o, double dflt = 0.0) {
  return o >= 0 ? *reinterpret_cast<const double*>(r + o) : dflt;
}
__device__ __forceinline__ int rec_i(const unsigned char* r, int64_t o, int dflt = 0) {
  return o >= 0 ? *reinterpret_cast<const int*>(r + o) : dflt;
}

// Records -> input-order device arrays.  With state: the flags (active bit), levels and the
// solved state of every particle (kept by the inactive ones) into the block-timestep state.
__global__ void k_unpack_aos(const unsigned char* base, int n, int64_t stride, gsph_field_offsets off, OutPtrs o,
                             KdkState s, int with_state) {
  double* const* dst = o.p;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const unsigned char* r = base + (size_t) i * stride;
    const double* pr = reinterpret_cast<const double*>(r + off.r);
    const double* pv = reinterpret_cast<const double*>(r + off.v);
    dst[0][i] = pr[0]; dst[1][i] = pr[1]; dst[2][i] = pr[2];
    dst[3][i] = pv[0]; dst[4][i] = pv[1]; dst[5][i] = pv[2];
    dst[6][i] = *reinterpret_cast<const double*>(r + off.m);
    dst[7][i] = *reinterpret_cast<const double*>(r + off.u);
    dst[8][i] = *reinterpret_cast<const double*>(r + off.h);
    if (!with_state) continue;
    s.flags[i] = (rec_i(r, off.flags) & (int) GSPH_FLAG_ACTIVE) ? kFlagActive : (unsigned char) 0;
    s.level[i] = rec_i(r, off.level);
    s.levelneib[i] = rec_i(r, off.levelneib);
    // keep[] order: rho invomega zeta hfactor hrangesqd pressure sound ax ay az agx agy agz
    // gpot dudt div_v gpot_hydro (integrate.cuh)
    const int64_t ko[kKeep] = {off.rho, off.invomega, off.zeta, off.hfactor, off.hrangesqd, off.pressure, off.sound,
                               off.a, off.a >= 0 ? off.a + 8 : -1, off.a >= 0 ? off.a + 16 : -1,
                               off.atree, off.atree >= 0 ? off.atree + 8 : -1, off.atree >= 0 ? off.atree + 16 : -1,
                               off.gpot, off.dudt, off.div_v, off.gpot_hydro};
#pragma unroll
    for (int q = 0; q < kKeep; q++) s.keep[q][i] = rec_d(r, ko[q], q == 1 ? 1.0 : 0.0);
  }
}

// Flags and levels only (the records after CheckTimesteps), input order.
__global__ void k_unpack_flags(const unsigned char* base, int n, int64_t stride, gsph_field_offsets off, KdkState s) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const unsigned char* r = base + (size_t) i * stride;
    s.flags[i] = (rec_i(r, off.flags) & (int) GSPH_FLAG_ACTIVE) ? kFlagActive : (unsigned char) 0;
    s.level[i] = rec_i(r, off.level);
  }
}

struct FieldPtrs { const double* f[kNumFields]; };

// The output fields one write-back stores: leaf-order field index and byte offset.
constexpr int kMaxOut = 24;
struct OutTable {
  int nf;
  int fidx[kMaxOut];
  int64_t foff[kMaxOut];
};

// Results straight into page-locked host records (device-visible address), slot order.
__global__ void k_write_aos_direct(unsigned char* base, int n, int64_t stride, OutTable t, FieldPtrs fp,
                                   const int* __restrict__ id, const unsigned char* __restrict__ active,
                                   const int* __restrict__ lvn, int64_t off_lvn) {
  for (int sl = blockIdx.x * blockDim.x + threadIdx.x; sl < n; sl += gridDim.x * blockDim.x) {
    unsigned char* r = base + (size_t) id[sl] * stride;
    if (lvn && off_lvn >= 0) {
      int* L = reinterpret_cast<int*>(r + off_lvn);
      const int v = lvn[sl];
      if (v > *L) *L = v;
    }
    if (active && !active[sl]) continue;
    for (int q = 0; q < t.nf; q++) *reinterpret_cast<double*>(r + t.foff[q]) = fp.f[t.fidx[q]][sl];
  }
}

// Staged write-back: the output fields, the active flags and the neighbour levels in input
// order into one compact device buffer (fields x n doubles, then n ints, then n bytes).
__global__ void k_pack_out(int n, OutTable t, FieldPtrs fp, const int* __restrict__ slot_of,
                           const unsigned char* __restrict__ active, const int* __restrict__ lvn, double* out) {
  int* lv = reinterpret_cast<int*>(out + (size_t) t.nf * n);
  unsigned char* ac = reinterpret_cast<unsigned char*>(lv + n);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int sl = slot_of[i];
    for (int q = 0; q < t.nf; q++) out[(size_t) q * n + i] = fp.f[t.fidx[q]][sl];
    lv[i] = lvn ? lvn[sl] : 0;
    ac[i] = active ? active[sl] : (unsigned char) 1;
  }
}

// Leaf order -> input order, written in input order (coalesced stores, random loads).
__global__ void k_scatter_field(const double* __restrict__ src, const int* __restrict__ slot_of, int n, double* dst) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) dst[i] = src[slot_of[i]];
}

int field_index(const gsph_ctx* c, int field) {
  switch (field) {
    case GSPH_FIELD_GPOT_HYDRO: return c->nstar ? kFGpotHydro : kFGpot;
    case GSPH_FIELD_H: return kFH;
    case GSPH_FIELD_RHO: return kFRho;
    case GSPH_FIELD_INVOMEGA: return kFInvOmega;
    case GSPH_FIELD_ZETA: return kFZeta;
    case GSPH_FIELD_HFACTOR: return kFHfactor;
    case GSPH_FIELD_PRESSURE: return kFPressure;
    case GSPH_FIELD_SOUND: return kFSound;
    case GSPH_FIELD_U: return kFU;
    case GSPH_FIELD_DIV_V: return kFDivV;
    case GSPH_FIELD_DUDT: return kFDudt;
    case GSPH_FIELD_AX: return kFAX;
    case GSPH_FIELD_AY: return kFAY;
    case GSPH_FIELD_AZ: return kFAZ;
    case GSPH_FIELD_AGX: return kFAGX;
    case GSPH_FIELD_AGY: return kFAGY;
    case GSPH_FIELD_AGZ: return kFAGZ;
    case GSPH_FIELD_GPOT: return kFGpot;
    case GSPH_FIELD_HRANGESQD: return kFHrangesqd;
    default: return -1;
  }
}

int grid1(int n) { return std::max(1, std::min((n + 255) / 256, 152 * 8)); }

int check_launch(gsph_ctx* c, const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(c, e, what);
  return GSPH_OK;
}

int read_status(gsph_ctx* c) {
  unsigned long long h[6];
  GSPH_CUDA(cudaMemcpyAsync(h, c->counters, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
  GSPH_CUDA(cudaStreamSynchronize(c->stream));
  c->last.status = (uint32_t) h[0];
  c->last.launches = c->launches;
  {
    int hc[2] = {0, 0};
    GSPH_CUDA(cudaMemcpy(hc, c->heavy_count + 2, sizeof(hc), cudaMemcpyDeviceToHost));
    c->last.heavy_density = hc[0];
    c->last.heavy_forces = hc[1];
  }
  c->last.density_pairs = (int64_t) h[1];
  c->last.hydro_pairs = (int64_t) h[2];
  c->last.direct_pairs = (int64_t) h[3];
  c->last.cell_pairs = (int64_t) h[4];
  c->last.exact_checks = (int64_t) h[5];
  const unsigned st = (unsigned) h[0];
  if (st & kStatusHNotConverged) return fail(c, GSPH_ERR_NOT_CONVERGED, "Problem with convergence of h-rho iteration");
  if (st & kStatusStackOverflow) return fail(c, GSPH_ERR_CAPACITY, "tree walk stack overflow");
  if (st & kStatusRetryLimit) return fail(c, GSPH_ERR_CAPACITY, "hmax retry limit reached");
  if (st & kStatusPartitionWait) return fail(c, GSPH_ERR_CUDA, "tree build: a partition wait gave up");
  return GSPH_OK;
}

// Phase timestamps; inside a graph capture they become event-record nodes of the graph.
void mark(gsph_ctx* c, int q) {
  if (c->in_body) return;   // conditional graph bodies hold no event records
  if (c->capturing) cudaEventRecordWithFlags(c->ev[q], c->stream, cudaEventRecordExternal);
  else cudaEventRecord(c->ev[q], c->stream);
}

int do_build(gsph_ctx* c) {
  if (!c->have_particles) return fail(c, GSPH_ERR_STATE, "no particles imported");
  BuildArgs a{};
  a.n = c->n; a.ltot = c->ltot; a.P = c->P;
  a.in = InputArrays{c->in[0], c->in[1], c->in[2], c->in[3], c->in[4], c->in[5], c->in[6], c->in[7], c->in[8]};
  for (int q = 0; q < 3; q++) {
    a.sort.key[q] = c->key[q]; a.sort.idx[q] = c->idx[q]; a.lists_b[q] = c->listb[q]; a.key2[q] = c->key2[q];
  }
  a.radix_hist = c->radix_hist;
  a.radix_tot = c->radix_tot;
  a.deep_inv = c->deep_inv;
  a.side[0] = c->side; a.side[1] = c->side2; a.seg_axis = c->seg_axis; a.seg_axis_next = c->seg_axis_next;
  a.part = PartitionState{c->part_tiles, c->part_sync, c->part_sync + 1, reinterpret_cast<unsigned*>(c->counters)};
  a.rootkey = c->rootkey; a.ibox = c->ibox;
  a.heap_first = c->heap_first; a.heap_n = c->heap_n; a.heap_ones_before = c->heap_ones;
  a.p = make_particles(c);
  a.id_out = c->id;
  a.slot_of = c->slot_of;
  a.tree = make_tree(c);
  a.thetamaxsqd = c->cfg.thetamaxsqd;
  c->launches += (unsigned) launch_build_tree(a, c->stream);
  if (c->bactive) {
    // records with flags: active flags, levels and the solved state of every particle
    // into leaf order (the inactive particles keep theirs)
    launch_kdk_gather(make_kdk_state(c), make_kdk_leaf(c), c->kg, c->stream);
    c->launches += 1;
  }
  if (mixed(c)) {
    launch_mixed_prep_build(a.tree, a.p, make_mixed_particles(c), make_mixed_cells(c), c->stream);
    c->launches += 2;
  }
  c->have_tree = true;
  c->have_props = c->have_forces = false;
  c->keep_current = false;
  return check_launch(c, "build tree");
}

int do_props(gsph_ctx* c) {
  if (!c->have_tree) return fail(c, GSPH_ERR_STATE, "tree not built");
  const Tree t = make_tree(c);
  const Particles p = make_particles(c);
  HeavyList heavy{c->heavy_leaves, c->heavy_count};
  if (mixed(c)) {
    GSPH_CUDA(cudaMemsetAsync(c->heavy_count + 2, 0, 2 * sizeof(int), c->stream));
    c->launches += (unsigned) launch_density_mixed(t, p, make_mixed_particles(c), make_mixed_cells(c),
                                                   make_params(c), make_counters(c), heavy,
                                                   HeavyList{c->wide_leaves, c->heavy_count + 1}, c->lpg,
                                                   c->max_leaf, c->stream);
  } else {
    GSPH_CUDA(cudaMemsetAsync(c->heavy_count + 2, 0, 2 * sizeof(int), c->stream));
    launch_density(t, p, make_params(c), make_counters(c), heavy, c->lpg, c->dens_next, c->dens_comp, c->stream);
    c->launches += 2;
  }
  int rc = check_launch(c, "density");
  if (rc) return rc;
  GSPH_CUDA(cudaMemcpyAsync(c->heavy_count + 2, c->heavy_count, sizeof(int), cudaMemcpyDeviceToDevice, c->stream));
  mark(c, 2);
  c->launches += (unsigned) launch_update_hmax(t, p, c->stream);
  if (c->kdk || c->bactive) {   // every particle's thermal properties before the force pass
    launch_kdk_thermal(p, make_params(c), c->stream);
    c->launches += 1;
  }
  if (mixed(c)) {
    launch_mixed_prep_hydro(t, p, make_mixed_particles(c), make_mixed_cells(c), c->stream);
    c->launches += 2;
  }
  c->have_props = true;
  return check_launch(c, "update hmax");
}

int do_forces(gsph_ctx* c, bool gravity) {
  if (!c->have_props) return fail(c, GSPH_ERR_STATE, "smoothing lengths not solved");
  const Tree t = make_tree(c);
  const Particles p = make_particles(c);
  if (c->record && c->rec_sph_cnt) {
    GSPH_CUDA(cudaMemsetAsync(c->rec_sph_cnt, 0, sizeof(int) * (size_t) c->n, c->stream));
    GSPH_CUDA(cudaMemsetAsync(c->rec_dir_cnt, 0, sizeof(unsigned long long) * (size_t) c->n, c->stream));
    GSPH_CUDA(cudaMemsetAsync(c->rec_dir_hash, 0, sizeof(unsigned long long) * (size_t) c->n, c->stream));
    GSPH_CUDA(cudaMemsetAsync(c->rec_cell_cnt, 0, sizeof(unsigned long long) * (size_t) c->nleaf, c->stream));
    GSPH_CUDA(cudaMemsetAsync(c->rec_cell_hash, 0, sizeof(unsigned long long) * (size_t) c->nleaf, c->stream));
    if (c->rec_dir_max > 0 && c->rec_dir_n) {
      GSPH_CUDA(cudaMemsetAsync(c->rec_dir_n, 0, sizeof(int) * (size_t) c->n, c->stream));
      GSPH_CUDA(cudaMemsetAsync(c->rec_cell_n, 0, sizeof(int) * (size_t) c->nleaf, c->stream));
    }
  }
  HeavyList heavy{c->heavy_leaves, c->heavy_count};
  if (mixed(c)) {
    if (gravity) {
      c->launches += (unsigned) launch_all_forces_mixed(t, p, make_mixed_particles(c), make_mixed_cells(c),
                                                        make_params(c), make_counters(c), heavy, c->lpg,
                                                        c->max_leaf, c->stream);
      GSPH_CUDA(cudaMemcpyAsync(c->heavy_count + 3, c->heavy_count, sizeof(int), cudaMemcpyDeviceToDevice, c->stream));
    }
    else
      c->launches += (unsigned) launch_hydro_mixed(t, p, make_mixed_particles(c), make_mixed_cells(c),
                                                   make_params(c), make_counters(c), c->lpg, c->stream);
  } else {
    if (gravity) launch_all_forces(t, p, make_params(c), make_counters(c), c->lpg, c->stream);
    else launch_hydro_forces(t, p, make_params(c), make_counters(c), c->lpg, c->stream);
    c->launches += 2;
  }
  // star gravity on the gas, after gpot_hydro is taken (GradhSphTree.cpp:596-606)
  c->launches += (unsigned) (mixed(c) ? launch_gas_from_stars_mixed(p, make_mixed_particles(c), make_stars(c), c->stream)
                                      : launch_gas_from_stars(p, make_stars(c), c->stream));
  c->have_forces = true;
  c->have_star_forces = false;
  return check_launch(c, "forces");
}

int do_star_gas(gsph_ctx* c) {
  if (!c->have_props) return fail(c, GSPH_ERR_STATE, "smoothing lengths not solved");
  c->launches += (unsigned) launch_stars_from_gas(make_tree(c), make_particles(c), make_stars(c), make_params(c),
                                                  make_counters(c), c->max_leaf, c->stream);
  c->have_star_forces = true;
  return check_launch(c, "star gas forces");
}

int begin_counters(gsph_ctx* c) {
  c->launches = 0;
  GSPH_CUDA(cudaMemsetAsync(c->counters, 0, 16 * sizeof(unsigned long long), c->stream));
  return GSPH_OK;
}

int ensure_full_lists(gsph_ctx* c);

int ensure_recording(gsph_ctx* c) {
  if (!c->record) return GSPH_OK;
  const size_t need = (size_t) c->n * (sizeof(int) * (1 + c->rec_max) + 2 * sizeof(unsigned long long)) +
                      (size_t) c->nleaf * 2 * sizeof(unsigned long long);
  if (c->rec_sph_cnt && c->rec_bytes >= need) return ensure_full_lists(c);
  drop_graph(c);   // a captured step holds the old recording buffers
  drop_kdk_graph(c);
  int rc = alloc(c, c->rec_sph_cnt, c->n);
  if (!rc) rc = alloc(c, c->rec_sph_ids, (size_t) c->n * c->rec_max);
  if (!rc) rc = alloc(c, c->rec_dir_cnt, c->n);
  if (!rc) rc = alloc(c, c->rec_dir_hash, c->n);
  if (!rc) rc = alloc(c, c->rec_cell_cnt, c->nleaf);
  if (!rc) rc = alloc(c, c->rec_cell_hash, c->nleaf);
  if (rc) return rc;
  c->rec_bytes = need;
  return ensure_full_lists(c);
}

// Full-list buffers for the current particle count (gsph_set_list_recording).
int ensure_full_lists(gsph_ctx* c) {
  if (!c->record || c->rec_dir_max <= 0) return GSPH_OK;
  const size_t need = (size_t) c->n * (1 + (size_t) c->rec_dir_max) + (size_t) c->nleaf * (1 + (size_t) c->rec_cell_max);
  if (c->rec_dir_n && c->rec_full_bytes >= need) return GSPH_OK;
  drop_graph(c);
  drop_kdk_graph(c);
  int rc = alloc(c, c->rec_dir_n, c->n);
  if (!rc) rc = alloc(c, c->rec_dir_ids, (size_t) c->n * c->rec_dir_max);
  if (!rc) rc = alloc(c, c->rec_cell_n, c->nleaf);
  if (!rc) rc = alloc(c, c->rec_cell_ids, (size_t) c->nleaf * c->rec_cell_max);
  if (rc) return rc;
  c->rec_full_bytes = need;
  return GSPH_OK;
}

// A new particle set through the structure-of-arrays imports: every particle active, and
// any KDK integration must be set up again.
void leave_flag_mode(gsph_ctx* c) {
  if (c->bactive) drop_graph(c);
  c->bactive = false;
  c->kdk = false;
}

// Device-visible address of host records [p, p + bytes) when they lie in one page-locked
// (or managed) allocation; nullptr when the records must be staged through a copy.
unsigned char* device_view(const void* p, size_t bytes) {
  cudaPointerAttributes a0{}, a1{};
  const unsigned char* q = static_cast<const unsigned char*>(p);
  if (cudaPointerGetAttributes(&a0, q) != cudaSuccess || cudaPointerGetAttributes(&a1, q + bytes - 1) != cudaSuccess) {
    (void) cudaGetLastError();
    return nullptr;
  }
  if (a0.type == cudaMemoryTypeManaged && a1.type == cudaMemoryTypeManaged) return const_cast<unsigned char*>(q);
  if (a0.type != cudaMemoryTypeHost || a1.type != cudaMemoryTypeHost || !a0.devicePointer || !a1.devicePointer)
    return nullptr;
  unsigned char* d0 = static_cast<unsigned char*>(a0.devicePointer);
  unsigned char* d1 = static_cast<unsigned char*>(a1.devicePointer);
  return (d1 - d0 == (std::ptrdiff_t) (bytes - 1)) ? d0 : nullptr;
}

// Checks shared by the record imports and exports.
int check_offsets(gsph_ctx* c, int64_t n, int64_t stride, const gsph_field_offsets* off, bool need_flags) {
  if (n < 1 || n > (int64_t) 1 << 30 || stride < 8 || (stride % 8) != 0)
    return fail(c, GSPH_ERR_INVALID, "bad array-of-structures description");
  const int64_t ins[5] = {off->r, off->v, off->m, off->h, off->u};
  for (int q = 0; q < 5; q++)
    if (ins[q] < 0 || ins[q] % 8 != 0 || ins[q] + (q < 2 ? 24 : 8) > stride)
      return fail(c, GSPH_ERR_INVALID, "input field offset outside the record or misaligned");
  const int64_t outs[] = {off->rho, off->invomega, off->zeta, off->hfactor, off->hrangesqd, off->pressure,
                          off->sound, off->div_v, off->dudt, off->gpot, off->gpot_hydro};
  for (int64_t o : outs)
    if (o >= 0 && (o % 8 != 0 || o + 8 > stride)) return fail(c, GSPH_ERR_INVALID, "output offset outside the record");
  for (int64_t o : {off->a, off->atree})
    if (o >= 0 && (o % 8 != 0 || o + 24 > stride)) return fail(c, GSPH_ERR_INVALID, "output offset outside the record");
  for (int64_t o : {off->flags, off->level, off->levelneib})
    if (o >= 0 && (o % 4 != 0 || o + 4 > stride)) return fail(c, GSPH_ERR_INVALID, "integer field offset outside the record");
  if (need_flags && off->flags < 0) return fail(c, GSPH_ERR_INVALID, "the records' flags offset is needed");
  return GSPH_OK;
}

}  // namespace

// ======================================================================================
extern "C" {

int32_t gsph_abi_version(void) { return GSPH_ABI_VERSION; }

void gsph_config_defaults(gsph_config* cfg) {
  if (!cfg) return;
  std::memset(cfg, 0, sizeof(*cfg));
  cfg->ndim = 3;
  cfg->nleafmax = 8;
  cfg->hydro_forces = 1;
  cfg->self_gravity = 0;
  cfg->eos = GSPH_EOS_ENERGY_EQN;
  cfg->multipole = GSPH_QUADRUPOLE;
  cfg->periodic = 0;
  cfg->precision = GSPH_PRECISION_FP64;
  cfg->h_fac = 1.2;
  cfg->h_converge = 0.01;
  cfg->alpha_visc = 1.0;
  cfg->beta_visc = 2.0;
  cfg->gamma_eos = 1.66666666666666;
  cfg->temp0 = 1.0;
  cfg->mu_bar = 1.0;
  cfg->thetamaxsqd = 0.1;
  for (int k = 0; k < 3; k++) { cfg->boxmin[k] = 0.0; cfg->boxmax[k] = 1.0; }
}

int32_t gsph_create_error(void) { return g_create_error; }

gsph_ctx* gsph_create(const gsph_config* cfg, int32_t device) {
  std::string why;
  const int rc = check_config(cfg, why);
  if (rc != GSPH_OK) { g_create_error = rc; return nullptr; }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
    g_create_error = GSPH_ERR_CUDA;
    return nullptr;
  }
  if (cudaSetDevice(device) != cudaSuccess) { g_create_error = GSPH_ERR_CUDA; return nullptr; }
  gsph_ctx* c = new gsph_ctx();
  c->cfg = *cfg;
  c->device = device;
  if (cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete c;
    g_create_error = GSPH_ERR_CUDA;
    return nullptr;
  }
  c->stream = c->own_stream;
  for (int q = 0; q < 5; q++) cudaEventCreate(&c->ev[q]);
  g_create_error = GSPH_OK;
  return c;
}

void gsph_destroy(gsph_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  drop_graph(c);
  kdk_free(c);
  free_all(c);
  if (c->aos) cudaFree(c->aos);
  if (c->aos_out) cudaFree(c->aos_out);
  if (c->kdk_snap) cudaFree(c->kdk_snap);
  for (int q = 0; q < 2; q++) if (c->cond_stream[q]) cudaStreamDestroy(c->cond_stream[q]);
  if (c->star_buf) cudaFree(c->star_buf);
  if (c->star_f) cudaFree(c->star_f);
  for (int q = 0; q < 5; q++) if (c->ev[q]) cudaEventDestroy(c->ev[q]);
  if (c->own_stream) cudaStreamDestroy(c->own_stream);
  delete c;
}

int32_t gsph_set_stream(gsph_ctx* c, void* stream) {
  if (!c) return GSPH_ERR_INVALID;
  cudaSetDevice(c->device);
  GSPH_CUDA(cudaStreamSynchronize(c->stream));
  c->stream = stream ? static_cast<cudaStream_t>(stream) : c->own_stream;
  return GSPH_OK;
}

const char* gsph_last_error(const gsph_ctx* c) { return c ? c->err.c_str() : "null context"; }

int32_t gsph_set_particles(gsph_ctx* c, int64_t n, const double* x, const double* y, const double* z,
                           const double* vx, const double* vy, const double* vz, const double* m,
                           const double* u, const double* h) {
  if (!c) return GSPH_ERR_INVALID;
  if (n < 1 || n > (int64_t) 1 << 30) return fail(c, GSPH_ERR_INVALID, "particle count out of range");
  cudaSetDevice(c->device);
  const double* a[9] = {x, y, z, vx, vy, vz, m, u, h};
  int rc = validate_host(c, n, a);
  if (rc) return rc;
  rc = ensure_capacity(c, (int) n);
  if (rc) return rc;
  for (int q = 0; q < 9; q++)
    GSPH_CUDA(cudaMemcpyAsync(c->in[q], a[q], sizeof(double) * (size_t) n, cudaMemcpyHostToDevice, c->stream));
  leave_flag_mode(c);
  c->have_particles = true;
  c->have_tree = c->have_props = c->have_forces = false;
  return GSPH_OK;
}

int32_t gsph_set_particles_device(gsph_ctx* c, int64_t n, const double* x, const double* y, const double* z,
                                  const double* vx, const double* vy, const double* vz, const double* m,
                                  const double* u, const double* h) {
  if (!c) return GSPH_ERR_INVALID;
  if (n < 1 || n > (int64_t) 1 << 30) return fail(c, GSPH_ERR_INVALID, "particle count out of range");
  const double* a[9] = {x, y, z, vx, vy, vz, m, u, h};
  for (int q = 0; q < 9; q++) if (!a[q]) return fail(c, GSPH_ERR_INVALID, "particle array is NULL");
  cudaSetDevice(c->device);
  int rc = ensure_capacity(c, (int) n);
  if (rc) return rc;
  for (int q = 0; q < 9; q++)
    GSPH_CUDA(cudaMemcpyAsync(c->in[q], a[q], sizeof(double) * (size_t) n, cudaMemcpyDeviceToDevice, c->stream));
  leave_flag_mode(c);
  c->have_particles = true;
  c->have_tree = c->have_props = c->have_forces = false;
  return GSPH_OK;
}

int32_t gsph_set_particles_aos(gsph_ctx* c, const void* base, int64_t n, int64_t stride, const gsph_field_offsets* off) {
  if (!c) return GSPH_ERR_INVALID;
  if (!base || !off) return fail(c, GSPH_ERR_INVALID, "bad array-of-structures description");
  int rc = check_offsets(c, n, stride, off, false);
  if (rc) return rc;
  cudaSetDevice(c->device);
  rc = ensure_capacity(c, (int) n);
  if (rc) return rc;
  const bool flags = off->flags >= 0;
  if (flags) {
    rc = ensure_kdk_buffers(c);
    if (rc) return rc;
  }
  if (flags != c->bactive) drop_graph(c);   // the step graph gathers the state only with flags
  c->bactive = flags;
  c->kdk = false;
  const size_t bytes = (size_t) n * (size_t) stride;
  const unsigned char* src = device_view(base, bytes);
  if (!src) {   // pageable records: one copy of the whole array, unpacked on the device
    if (bytes > c->aos_bytes) {
      if (c->aos) cudaFree(c->aos);
      c->aos = nullptr;
      c->aos_bytes = 0;
      GSPH_CUDA(cudaMalloc(&c->aos, bytes));
      c->aos_bytes = bytes;
    }
    GSPH_CUDA(cudaMemcpyAsync(c->aos, base, bytes, cudaMemcpyHostToDevice, c->stream));
    src = static_cast<const unsigned char*>(c->aos);
  }
  c->aos_stride = stride;
  OutPtrs o;
  for (int q = 0; q < 9; q++) o.p[q] = c->in[q];
  KdkState ks{};
  if (flags) ks = make_kdk_state(c);
  k_unpack_aos<<<grid1((int) n), 256, 0, c->stream>>>(src, (int) n, stride, *off, o, ks, flags ? 1 : 0);
  rc = check_launch(c, "unpack");
  if (rc) return rc;
  if (src != c->aos) GSPH_CUDA(cudaStreamSynchronize(c->stream));   // the caller may change the records
  c->have_particles = true;
  c->have_tree = c->have_props = c->have_forces = false;
  return GSPH_OK;
}

int32_t gsph_update_active_particle_counters(gsph_ctx* c, const void* base, int64_t n, int64_t stride,
                                             const gsph_field_offsets* off) {
  if (!c) return GSPH_ERR_INVALID;
  if (!base || !off) return fail(c, GSPH_ERR_INVALID, "bad array-of-structures description");
  int rc = check_offsets(c, n, stride, off, true);
  if (rc) return rc;
  if (!c->bactive || n != c->n || stride != c->aos_stride)
    return fail(c, GSPH_ERR_STATE, "records with flags were not imported with gsph_set_particles_aos");
  if (!c->have_tree) return fail(c, GSPH_ERR_STATE, "tree not built");
  cudaSetDevice(c->device);
  const size_t bytes = (size_t) n * (size_t) stride;
  const unsigned char* src = device_view(base, bytes);
  if (!src) {
    if (bytes > c->aos_bytes) return fail(c, GSPH_ERR_STATE, "record staging buffer too small");
    GSPH_CUDA(cudaMemcpyAsync(c->aos, base, bytes, cudaMemcpyHostToDevice, c->stream));
    src = static_cast<const unsigned char*>(c->aos);
  }
  const KdkState ks = make_kdk_state(c);
  k_unpack_flags<<<grid1((int) n), 256, 0, c->stream>>>(src, (int) n, stride, *off, ks);
  launch_kdk_refresh(ks, make_kdk_leaf(c), c->kg, c->stream);   // leaf-order flags, levels; levelneib restarts
  rc = check_launch(c, "update active counters");
  if (rc) return rc;
  GSPH_CUDA(cudaStreamSynchronize(c->stream));
  c->have_props = c->have_forces = false;
  return GSPH_OK;
}

int32_t gsph_get_maximum_smoothing_length(gsph_ctx* c, double* hmax) {
  if (!c || !hmax) return GSPH_ERR_INVALID;
  if (!c->have_tree) return fail(c, GSPH_ERR_STATE, "tree not built");
  cudaSetDevice(c->device);
  CellGeom g{};
  GSPH_CUDA(cudaMemcpyAsync(&g, c->geom, sizeof(g), cudaMemcpyDeviceToHost, c->stream));
  GSPH_CUDA(cudaStreamSynchronize(c->stream));
  *hmax = g.hmax;
  return GSPH_OK;
}

int32_t gsph_build_tree(gsph_ctx* c) {
  if (!c) return GSPH_ERR_INVALID;
  cudaSetDevice(c->device);
  int rc = begin_counters(c);
  if (rc) return rc;
  rc = do_build(c);
  if (rc) return rc;
  GSPH_CUDA(cudaStreamSynchronize(c->stream));
  return GSPH_OK;
}

int32_t gsph_update_all_sph_properties(gsph_ctx* c) {
  if (!c) return GSPH_ERR_INVALID;
  cudaSetDevice(c->device);
  int rc = begin_counters(c);
  if (rc) return rc;
  rc = do_props(c);
  if (rc) return rc;
  return read_status(c);
}

int32_t gsph_update_all_sph_hydro_forces(gsph_ctx* c) {
  if (!c) return GSPH_ERR_INVALID;
  cudaSetDevice(c->device);
  int rc = ensure_recording(c);
  if (rc) return rc;
  rc = begin_counters(c);
  if (rc) return rc;
  rc = do_forces(c, false);
  if (rc) return rc;
  return read_status(c);
}

int32_t gsph_update_all_sph_forces(gsph_ctx* c) {
  if (!c) return GSPH_ERR_INVALID;
  if (!c->cfg.self_gravity) return fail(c, GSPH_ERR_STATE, "self_gravity is off in this context");
  cudaSetDevice(c->device);
  int rc = ensure_recording(c);
  if (rc) return rc;
  rc = begin_counters(c);
  if (rc) return rc;
  rc = do_forces(c, true);
  if (rc) return rc;
  return read_status(c);
}

namespace {

// Everything one step launches, in stream order, with no host synchronisation (so that it
// can also be captured into a graph).
int step_body(gsph_ctx* c) {
  int rc = begin_counters(c);
  if (rc) return rc;
  mark(c, 0);
  rc = do_build(c);
  if (rc) return rc;
  mark(c, 1);
  rc = do_props(c);
  if (rc) return rc;
  mark(c, 3);
  rc = do_forces(c, c->cfg.self_gravity != 0);
  if (rc) return rc;
  if (c->nstar && c->cfg.self_gravity) {
    rc = do_star_gas(c);
    if (rc) return rc;
  }
  mark(c, 4);
  return GSPH_OK;
}

int finish_step(gsph_ctx* c) {
  const int rc = read_status(c);
  float ms[4] = {0, 0, 0, 0};
  for (int q = 0; q < 4; q++) {
    const int a = q, b = q + 1;
    if (cudaEventElapsedTime(&ms[q], c->ev[a], c->ev[b]) != cudaSuccess) ms[q] = 0.0f;
  }
  (void) cudaGetLastError();   // a phase event that was not recorded leaves no error behind
  c->last.ms_build = ms[0]; c->last.ms_density = ms[1]; c->last.ms_hmax = ms[2]; c->last.ms_forces = ms[3];
  c->last.ms_total = ms[0] + ms[1] + ms[2] + ms[3];
  return rc;
}

}  // namespace

int32_t gsph_step(gsph_ctx* c) {
  if (!c) return GSPH_ERR_INVALID;
  cudaSetDevice(c->device);
  int rc = ensure_recording(c);
  if (rc) return rc;
  rc = step_body(c);
  if (rc) return rc;
  return finish_step(c);
}

int32_t gsph_step_graph(gsph_ctx* c) {
  if (!c) return GSPH_ERR_INVALID;
  if (!c->have_particles) return fail(c, GSPH_ERR_STATE, "no particles imported");
  cudaSetDevice(c->device);
  int rc = ensure_recording(c);
  if (rc) return rc;
  if (!c->graph_valid) {
    drop_graph(c);
    // capture on the context's own stream (a caller's stream may be the legacy default
    // stream, which cannot be captured); the graph is launched on the current stream
    GSPH_CUDA(cudaStreamSynchronize(c->stream));
    cudaStream_t saved = c->stream;
    c->stream = c->own_stream;
    GSPH_CUDA(cudaStreamBeginCapture(c->own_stream, cudaStreamCaptureModeRelaxed));
    c->capturing = true;
    rc = step_body(c);
    c->capturing = false;
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(c->own_stream, &g);
    c->stream = saved;
    if (rc) { if (g) cudaGraphDestroy(g); return rc; }
    if (e != cudaSuccess) return cuda_fail(c, e, "cudaStreamEndCapture");
    c->graph = g;
    GSPH_CUDA(cudaGraphInstantiate(&c->graph_exec, c->graph, 0));
    c->graph_launches = c->launches;
    c->graph_valid = true;
  }
  GSPH_CUDA(cudaGraphLaunch(c->graph_exec, c->stream));
  c->launches = c->graph_launches;
  c->have_tree = c->have_props = c->have_forces = true;
  c->have_star_forces = c->nstar && c->cfg.self_gravity;
  return finish_step(c);
}

int32_t gsph_set_stars(gsph_ctx* c, int64_t nstar, const double* x, const double* y, const double* z,
                       const double* vx, const double* vy, const double* vz, const double* m, const double* h) {
  if (!c) return GSPH_ERR_INVALID;
  if (nstar < 0 || nstar > (1 << 20)) return fail(c, GSPH_ERR_INVALID, "star count out of range");
  const double* a[8] = {x, y, z, vx, vy, vz, m, h};
  if (nstar > 0) {
    for (int q = 0; q < 8; q++) if (!a[q]) return fail(c, GSPH_ERR_INVALID, "star array is NULL");
    for (int64_t i = 0; i < nstar; i++) {
      for (int q = 0; q < 8; q++)
        if (!std::isfinite(a[q][i])) return fail(c, GSPH_ERR_INVALID, "non-finite star data");
      if (!(m[i] > 0.0) || !(h[i] > 0.0)) return fail(c, GSPH_ERR_INVALID, "star mass and h must be > 0");
    }
  }
  cudaSetDevice(c->device);
  GSPH_CUDA(cudaStreamSynchronize(c->stream));
  if (nstar > c->star_cap) {
    drop_graph(c);
    if (c->star_buf) cudaFree(c->star_buf);
    if (c->star_f) cudaFree(c->star_f);
    c->star_buf = nullptr;
    c->star_f = nullptr;
    c->star_cap = 0;
    GSPH_CUDA(cudaMalloc(&c->star_buf, sizeof(double) * 15 * (size_t) nstar));
    GSPH_CUDA(cudaMalloc(&c->star_f, sizeof(float4) * 2 * (size_t) nstar));
    c->star_cap = (int) nstar;
  }
  for (int q = 0; q < 8 && nstar > 0; q++)
    GSPH_CUDA(cudaMemcpyAsync(c->star_buf + (size_t) q * c->star_cap, a[q], sizeof(double) * (size_t) nstar,
                              cudaMemcpyHostToDevice, c->stream));
  if (nstar > 0) {
    // positions as unevaluated float sums hi + lo (as the gas mirrors), mass and h
    c->star_f_host.assign(2 * (size_t) c->star_cap, make_float4(0.f, 0.f, 0.f, 0.f));
    for (int64_t i = 0; i < nstar; i++) {
      float hi[3], lo[3];
      const double r[3] = {x[i], y[i], z[i]};
      for (int k = 0; k < 3; k++) { hi[k] = (float) r[k]; lo[k] = (float) (r[k] - (double) hi[k]); }
      c->star_f_host[i] = make_float4(hi[0], hi[1], hi[2], (float) m[i]);
      c->star_f_host[c->star_cap + i] = make_float4(lo[0], lo[1], lo[2], (float) h[i]);
    }
    GSPH_CUDA(cudaMemcpyAsync(c->star_f, c->star_f_host.data(), sizeof(float4) * 2 * (size_t) c->star_cap,
                              cudaMemcpyHostToDevice, c->stream));
    GSPH_CUDA(cudaStreamSynchronize(c->stream));   // the staging vector may change before a later copy
  }
  if ((int) nstar != c->nstar || nstar > c->star_cap) drop_graph(c);
  c->nstar = (int) nstar;
  // the h solve (zeta term) and both force passes depend on the stars
  c->have_props = c->have_forces = c->have_star_forces = false;
  return GSPH_OK;
}

int32_t gsph_update_all_star_gas_forces(gsph_ctx* c) {
  if (!c) return GSPH_ERR_INVALID;
  if (!c->cfg.self_gravity) return fail(c, GSPH_ERR_STATE, "self_gravity is off in this context");
  if (!c->nstar) return fail(c, GSPH_ERR_STATE, "no star particles set");
  cudaSetDevice(c->device);
  int rc = begin_counters(c);
  if (rc) return rc;
  rc = do_star_gas(c);
  if (rc) return rc;
  return read_status(c);
}

int32_t gsph_get_star_forces(gsph_ctx* c, double* ax, double* ay, double* az, double* adotx, double* adoty,
                             double* adotz, double* gpot) {
  if (!c) return GSPH_ERR_INVALID;
  if (!c->have_star_forces) return fail(c, GSPH_ERR_STATE, "star <- gas forces not computed");
  cudaSetDevice(c->device);
  GSPH_CUDA(cudaStreamSynchronize(c->stream));
  double* out[7] = {ax, ay, az, adotx, adoty, adotz, gpot};
  const double* src = c->star_buf + 8 * (size_t) c->star_cap;
  for (int q = 0; q < 7; q++)
    if (out[q])
      GSPH_CUDA(cudaMemcpy(out[q], src + (size_t) q * c->star_cap, sizeof(double) * (size_t) c->nstar,
                           cudaMemcpyDeviceToHost));
  return GSPH_OK;
}

int32_t gsph_get_field_device(gsph_ctx* c, int32_t field, double* out) {
  if (!c || !out) return GSPH_ERR_INVALID;
  const int fi = field_index(c, field);
  if (fi < 0) return fail(c, GSPH_ERR_INVALID, "unknown field");
  if (!c->have_tree) return fail(c, GSPH_ERR_STATE, "no results yet");
  cudaSetDevice(c->device);
  if (c->kdk && c->keep_current) {
    // after KDK steps every particle's fields are in the integration state, input order
    // (the leaf-order arrays hold only what the last passes solved)
    const double* src = kdk_field_source(c, fi);
    if (src) {
      GSPH_CUDA(cudaMemcpyAsync(out, src, sizeof(double) * (size_t) c->n, cudaMemcpyDeviceToDevice, c->stream));
      return GSPH_OK;
    }
  }
  k_scatter_field<<<grid1(c->n), 256, 0, c->stream>>>(c->f[fi], c->slot_of, c->n, out);
  return check_launch(c, "scatter field");
}

int32_t gsph_get_field(gsph_ctx* c, int32_t field, double* out) {
  if (!c || !out) return GSPH_ERR_INVALID;
  int rc = gsph_get_field_device(c, field, c->scratch_out);
  if (rc) return rc;
  GSPH_CUDA(cudaMemcpyAsync(out, c->scratch_out, sizeof(double) * (size_t) c->n, cudaMemcpyDeviceToHost, c->stream));
  GSPH_CUDA(cudaStreamSynchronize(c->stream));
  return GSPH_OK;
}

int32_t gsph_get_particles_aos(gsph_ctx* c, void* base, int64_t n, int64_t stride, const gsph_field_offsets* off) {
  if (!c || !base || !off) return GSPH_ERR_INVALID;
  int rc = check_offsets(c, n, stride, off, false);
  if (rc) return rc;
  if (!c->have_particles || n != c->n) return fail(c, GSPH_ERR_STATE, "record count differs from the imported set");
  if (c->bactive && off->flags < 0)
    return fail(c, GSPH_ERR_INVALID, "the particles were imported with flags: pass the same offsets");
  if (!c->have_tree) return fail(c, GSPH_ERR_STATE, "no results yet");
  cudaSetDevice(c->device);
  // the fields computed since the import
  OutTable t{};
  auto add = [&](int64_t o, int fld) {
    if (o >= 0 && t.nf < kMaxOut) { t.fidx[t.nf] = fld; t.foff[t.nf] = o; t.nf++; }
  };
  if (c->have_props) {
    add(off->h, kFH); add(off->u, kFU); add(off->rho, kFRho); add(off->invomega, kFInvOmega);
    add(off->zeta, kFZeta); add(off->hfactor, kFHfactor); add(off->hrangesqd, kFHrangesqd);
    add(off->pressure, kFPressure); add(off->sound, kFSound);
  }
  if (c->have_forces) {
    add(off->div_v, kFDivV); add(off->dudt, kFDudt); add(off->gpot, kFGpot);
    add(off->gpot_hydro, c->nstar ? kFGpotHydro : kFGpot);
    if (off->a >= 0) { add(off->a, kFAX); add(off->a + 8, kFAY); add(off->a + 16, kFAZ); }
    if (off->atree >= 0) { add(off->atree, kFAGX); add(off->atree + 8, kFAGY); add(off->atree + 16, kFAGZ); }
  }
  const unsigned char* act = c->bactive ? c->leaf_active : nullptr;
  const int* lvn = (c->bactive && c->have_forces && off->levelneib >= 0) ? c->leaf_lvn : nullptr;
  if (t.nf == 0 && !lvn) return GSPH_OK;
  FieldPtrs fp;
  for (int q = 0; q < kNumFields; q++) fp.f[q] = c->f[q];
  const size_t bytes = (size_t) n * (size_t) stride;
  unsigned char* dst = device_view(base, bytes);
  if (dst) {   // page-locked records: written in place, only the output fields
    k_write_aos_direct<<<grid1(c->n), 256, 0, c->stream>>>(dst, c->n, stride, t, fp, c->id, act, lvn, off->levelneib);
    rc = check_launch(c, "write records");
    if (rc) return rc;
    GSPH_CUDA(cudaStreamSynchronize(c->stream));
    return GSPH_OK;
  }
  // pageable records: compact buffer (fields, neighbour levels, active flags; input order)
  const size_t need = sizeof(double) * (size_t) t.nf * (size_t) n + (sizeof(int) + 1) * (size_t) n;
  if (need > c->aos_out_bytes) {
    if (c->aos_out) cudaFree(c->aos_out);
    c->aos_out = nullptr;
    c->aos_out_bytes = 0;
    GSPH_CUDA(cudaMalloc(&c->aos_out, need));
    c->aos_out_bytes = need;
  }
  k_pack_out<<<grid1(c->n), 256, 0, c->stream>>>(c->n, t, fp, c->slot_of, act, lvn, c->aos_out);
  rc = check_launch(c, "pack outputs");
  if (rc) return rc;
  std::vector<unsigned char> h(need);
  GSPH_CUDA(cudaMemcpyAsync(h.data(), c->aos_out, need, cudaMemcpyDeviceToHost, c->stream));
  GSPH_CUDA(cudaStreamSynchronize(c->stream));
  const double* fv = reinterpret_cast<const double*>(h.data());
  const int* lv = reinterpret_cast<const int*>(fv + (size_t) t.nf * n);
  const unsigned char* ac = reinterpret_cast<const unsigned char*>(lv + n);
  unsigned char* rec0 = static_cast<unsigned char*>(base);
  for (int64_t i = 0; i < n; i++) {
    unsigned char* r = rec0 + (size_t) i * (size_t) stride;
    if (lvn) {
      int cur;
      std::memcpy(&cur, r + off->levelneib, sizeof(int));
      if (lv[i] > cur) std::memcpy(r + off->levelneib, &lv[i], sizeof(int));
    }
    if (!ac[i]) continue;
    for (int q = 0; q < t.nf; q++) std::memcpy(r + t.foff[q], &fv[(size_t) q * n + i], sizeof(double));
  }
  return GSPH_OK;
}

int32_t gsph_get_stats(gsph_ctx* c, gsph_stats* out) {
  if (!c || !out) return GSPH_ERR_INVALID;
  *out = c->last;
  out->n = c->n; out->ncell = c->ncell; out->nleaf = c->nleaf; out->ltot = c->ltot;
  return GSPH_OK;
}

int32_t gsph_set_recording(gsph_ctx* c, int32_t enable, int32_t max_sph) {
  if (!c) return GSPH_ERR_INVALID;
  if (enable && (max_sph < 1 || max_sph > 4096)) return fail(c, GSPH_ERR_INVALID, "max_sph must be 1..4096");
  if ((enable ? 1 : 0) != c->record || (enable && max_sph != c->rec_max)) { drop_graph(c); drop_kdk_graph(c); }
  c->record = enable ? 1 : 0;
  if (enable && max_sph != c->rec_max) { c->rec_sph_cnt = nullptr; c->rec_bytes = 0; }
  c->rec_max = enable ? max_sph : 0;
  return GSPH_OK;
}

int64_t gsph_get_sph_neighbours(gsph_ctx* c, int64_t* offsets, int32_t* ids) {
  if (!c) return GSPH_ERR_INVALID;
  if (!c->record || !c->rec_sph_cnt || !c->have_forces) return fail(c, GSPH_ERR_STATE, "no recorded force pass");
  cudaSetDevice(c->device);
  const int n = c->n;
  std::vector<int> cntv(n), idv(n);
  std::vector<int> sids((size_t) n * c->rec_max);
  GSPH_CUDA(cudaMemcpy(cntv.data(), c->rec_sph_cnt, sizeof(int) * n, cudaMemcpyDeviceToHost));
  GSPH_CUDA(cudaMemcpy(idv.data(), c->id, sizeof(int) * n, cudaMemcpyDeviceToHost));
  GSPH_CUDA(cudaMemcpy(sids.data(), c->rec_sph_ids, sizeof(int) * sids.size(), cudaMemcpyDeviceToHost));
  std::vector<int64_t> cnt_in(n);
  int64_t total = 0;
  for (int s = 0; s < n; s++) {
    if (cntv[s] > c->rec_max) return fail(c, GSPH_ERR_CAPACITY, "recorded SPH list exceeded max_sph");
    cnt_in[idv[s]] = cntv[s];
    total += cntv[s];
  }
  if (!ids) return total;
  if (!offsets) return GSPH_ERR_INVALID;
  offsets[0] = 0;
  for (int i = 0; i < n; i++) offsets[i + 1] = offsets[i] + cnt_in[i];
  for (int s = 0; s < n; s++) {
    const int i = idv[s];
    for (int k = 0; k < cntv[s]; k++) ids[offsets[i] + k] = idv[sids[(size_t) s * c->rec_max + k]];
  }
  return total;
}

int32_t gsph_get_direct_summary(gsph_ctx* c, int64_t* counts, uint64_t* hashes) {
  if (!c || !counts || !hashes) return GSPH_ERR_INVALID;
  if (!c->record || !c->rec_sph_cnt || !c->have_forces) return fail(c, GSPH_ERR_STATE, "no recorded force pass");
  cudaSetDevice(c->device);
  const int n = c->n;
  std::vector<unsigned long long> dc(n), dh(n);
  std::vector<int> idv(n);
  GSPH_CUDA(cudaMemcpy(dc.data(), c->rec_dir_cnt, sizeof(unsigned long long) * n, cudaMemcpyDeviceToHost));
  GSPH_CUDA(cudaMemcpy(dh.data(), c->rec_dir_hash, sizeof(unsigned long long) * n, cudaMemcpyDeviceToHost));
  GSPH_CUDA(cudaMemcpy(idv.data(), c->id, sizeof(int) * n, cudaMemcpyDeviceToHost));
  for (int s = 0; s < n; s++) { counts[idv[s]] = (int64_t) dc[s]; hashes[idv[s]] = dh[s]; }
  return GSPH_OK;
}

int32_t gsph_get_cell_summary(gsph_ctx* c, int32_t* leaf_cells, int64_t* counts, uint64_t* hashes) {
  if (!c || !leaf_cells || !counts || !hashes) return GSPH_ERR_INVALID;
  if (!c->record || !c->rec_sph_cnt || !c->have_forces) return fail(c, GSPH_ERR_STATE, "no recorded force pass");
  cudaSetDevice(c->device);
  const int nl = c->nleaf;
  std::vector<unsigned long long> cc(nl), ch(nl);
  GSPH_CUDA(cudaMemcpy(leaf_cells, c->leaf_cell, sizeof(int) * nl, cudaMemcpyDeviceToHost));
  GSPH_CUDA(cudaMemcpy(cc.data(), c->rec_cell_cnt, sizeof(unsigned long long) * nl, cudaMemcpyDeviceToHost));
  GSPH_CUDA(cudaMemcpy(ch.data(), c->rec_cell_hash, sizeof(unsigned long long) * nl, cudaMemcpyDeviceToHost));
  for (int q = 0; q < nl; q++) { counts[q] = (int64_t) cc[q]; hashes[q] = ch[q]; }
  return GSPH_OK;
}

int32_t gsph_set_list_recording(gsph_ctx* c, int32_t max_direct, int32_t max_cells) {
  if (!c) return GSPH_ERR_INVALID;
  if (max_direct < 0 || max_cells < 0 || max_direct > (1 << 20) || max_cells > (1 << 20) ||
      (max_direct > 0) != (max_cells > 0))
    return fail(c, GSPH_ERR_INVALID, "list capacities must both be 0 or both in 1..2^20");
  if (max_direct != c->rec_dir_max || max_cells != c->rec_cell_max) {
    drop_graph(c);
    drop_kdk_graph(c);
    c->rec_dir_n = c->rec_dir_ids = c->rec_cell_n = c->rec_cell_ids = nullptr;   // reallocated on demand
    c->rec_full_bytes = 0;
  }
  c->rec_dir_max = max_direct;
  c->rec_cell_max = max_cells;
  return GSPH_OK;
}

int64_t gsph_get_direct_lists(gsph_ctx* c, int64_t* offsets, int32_t* ids) {
  if (!c) return GSPH_ERR_INVALID;
  if (!c->record || !c->rec_dir_n || !c->have_forces) return fail(c, GSPH_ERR_STATE, "no recorded force pass with full lists");
  cudaSetDevice(c->device);
  GSPH_CUDA(cudaStreamSynchronize(c->stream));
  const int n = c->n, mx = c->rec_dir_max;
  std::vector<int> cnt(n), idv(n), all((size_t) n * mx);
  GSPH_CUDA(cudaMemcpy(cnt.data(), c->rec_dir_n, sizeof(int) * n, cudaMemcpyDeviceToHost));
  GSPH_CUDA(cudaMemcpy(idv.data(), c->id, sizeof(int) * n, cudaMemcpyDeviceToHost));
  GSPH_CUDA(cudaMemcpy(all.data(), c->rec_dir_ids, sizeof(int) * all.size(), cudaMemcpyDeviceToHost));
  std::vector<int64_t> cin(n);
  int64_t total = 0;
  for (int s = 0; s < n; s++) {
    if (cnt[s] > mx) return fail(c, GSPH_ERR_CAPACITY, "a direct-sum list exceeded max_direct");
    cin[idv[s]] = cnt[s];
    total += cnt[s];
  }
  if (!ids) return total;
  if (!offsets) return GSPH_ERR_INVALID;
  offsets[0] = 0;
  for (int i = 0; i < n; i++) offsets[i + 1] = offsets[i] + cin[i];
  for (int s = 0; s < n; s++)
    for (int k = 0; k < cnt[s]; k++) ids[offsets[idv[s]] + k] = all[(size_t) s * mx + k];
  return total;
}

int64_t gsph_get_cell_lists(gsph_ctx* c, int64_t* offsets, int32_t* cells) {
  if (!c) return GSPH_ERR_INVALID;
  if (!c->record || !c->rec_cell_n || !c->have_forces) return fail(c, GSPH_ERR_STATE, "no recorded force pass with full lists");
  cudaSetDevice(c->device);
  GSPH_CUDA(cudaStreamSynchronize(c->stream));
  const int nl = c->nleaf, mx = c->rec_cell_max;
  std::vector<int> cnt(nl), all((size_t) nl * mx);
  GSPH_CUDA(cudaMemcpy(cnt.data(), c->rec_cell_n, sizeof(int) * nl, cudaMemcpyDeviceToHost));
  GSPH_CUDA(cudaMemcpy(all.data(), c->rec_cell_ids, sizeof(int) * all.size(), cudaMemcpyDeviceToHost));
  int64_t total = 0;
  for (int q = 0; q < nl; q++) {
    if (cnt[q] > mx) return fail(c, GSPH_ERR_CAPACITY, "a multipole-cell list exceeded max_cells");
    total += cnt[q];
  }
  if (!cells) return total;
  if (!offsets) return GSPH_ERR_INVALID;
  offsets[0] = 0;
  for (int q = 0; q < nl; q++) {
    offsets[q + 1] = offsets[q] + cnt[q];
    for (int k = 0; k < cnt[q]; k++) cells[offsets[q] + k] = all[(size_t) q * mx + k];
  }
  return total;
}

int32_t gsph_get_tree(gsph_ctx* c, int32_t* cell_n, int32_t* cell_first, int32_t* order, double* cell_data) {
  if (!c) return GSPH_ERR_INVALID;
  if (!c->have_tree) return fail(c, GSPH_ERR_STATE, "tree not built");
  cudaSetDevice(c->device);
  GSPH_CUDA(cudaStreamSynchronize(c->stream));
  const int nc = c->ncell;
  if (cell_n) GSPH_CUDA(cudaMemcpy(cell_n, c->cell_n, sizeof(int) * nc, cudaMemcpyDeviceToHost));
  if (cell_first) GSPH_CUDA(cudaMemcpy(cell_first, c->cell_first, sizeof(int) * nc, cudaMemcpyDeviceToHost));
  if (order) GSPH_CUDA(cudaMemcpy(order, c->id, sizeof(int) * c->n, cudaMemcpyDeviceToHost));
  if (cell_data) {
    std::vector<CellGeom> g(nc);
    std::vector<CellBox> b(nc), hb(nc);
    std::vector<CellMoment> mo(nc);
    std::vector<int> cn(nc), cf(nc);
    std::vector<unsigned char> lv(nc);
    GSPH_CUDA(cudaMemcpy(g.data(), c->geom, sizeof(CellGeom) * nc, cudaMemcpyDeviceToHost));
    GSPH_CUDA(cudaMemcpy(b.data(), c->bb, sizeof(CellBox) * nc, cudaMemcpyDeviceToHost));
    GSPH_CUDA(cudaMemcpy(hb.data(), c->hbox, sizeof(CellBox) * nc, cudaMemcpyDeviceToHost));
    GSPH_CUDA(cudaMemcpy(mo.data(), c->mom, sizeof(CellMoment) * nc, cudaMemcpyDeviceToHost));
    GSPH_CUDA(cudaMemcpy(cn.data(), c->cell_n, sizeof(int) * nc, cudaMemcpyDeviceToHost));
    GSPH_CUDA(cudaMemcpy(cf.data(), c->cell_first, sizeof(int) * nc, cudaMemcpyDeviceToHost));
    GSPH_CUDA(cudaMemcpy(lv.data(), c->cell_level, nc, cudaMemcpyDeviceToHost));
    for (int q = 0; q < nc; q++) {
      double* r = cell_data + (size_t) q * 31;
      r[0] = cn[q]; r[1] = lv[q]; r[2] = mo[q].m; r[3] = g[q].rmax; r[4] = g[q].hmax; r[5] = g[q].cdistsqd;
      for (int k = 0; k < 3; k++) {
        r[6 + k] = b[q].bbmin[k]; r[9 + k] = b[q].bbmax[k]; r[12 + k] = hb[q].bbmin[k]; r[15 + k] = hb[q].bbmax[k];
        r[18 + k] = g[q].rcell[k]; r[21 + k] = mo[q].r[k];
      }
      for (int k = 0; k < 5; k++) r[24 + k] = mo[q].q[k];
      r[29] = cf[q]; r[30] = 0;
    }
  }
  return GSPH_OK;
}

}  // extern "C"

// ======================================================================================
// Autotuning (gsph_get_tuning / gsph_set_tuning / gsph_autotune)
// ======================================================================================
extern "C" {

int32_t gsph_get_tuning(gsph_ctx* c, gsph_tuning* out) {
  if (!c || !out) return GSPH_ERR_INVALID;
  out->nleafmax = c->cfg.nleafmax;
  out->near_depth = c->near_depth;
  out->cell_depth = c->cell_depth;
  out->gather_depth = c->gather_depth;
  return GSPH_OK;
}

int32_t gsph_set_tuning(gsph_ctx* c, const gsph_tuning* t) {
  if (!c || !t) return GSPH_ERR_INVALID;
  if (t->nleafmax < 1 || t->nleafmax > 32) return fail(c, GSPH_ERR_INVALID, "nleafmax must be 1..32");
  if ((t->near_depth && (t->near_depth < 64 || t->near_depth > 256)) ||
      (t->cell_depth && (t->cell_depth < 64 || t->cell_depth > 512)) ||
      (t->gather_depth && (t->gather_depth < 64 || t->gather_depth > 256)))
    return fail(c, GSPH_ERR_INVALID, "depth outside its range");
  cudaSetDevice(c->device);
  if (t->nleafmax != c->cfg.nleafmax) {
    if (c->bactive) return fail(c, GSPH_ERR_STATE, "set the leaf size before importing records with flags");
    GSPH_CUDA(cudaStreamSynchronize(c->stream));
    const int n = c->n;
    double* save = nullptr;
    if (c->have_particles) {   // a new shape may reallocate the particle arrays: keep the inputs
      GSPH_CUDA(cudaMalloc(&save, sizeof(double) * 9 * (size_t) n));
      for (int q = 0; q < 9; q++)
        GSPH_CUDA(cudaMemcpyAsync(save + (size_t) q * n, c->in[q], sizeof(double) * n, cudaMemcpyDeviceToDevice,
                                  c->stream));
    }
    const int old = c->cfg.nleafmax;
    c->cfg.nleafmax = t->nleafmax;
    int rc = GSPH_OK;
    if (c->have_particles) {
      c->have_particles = false;   // recompute the tree shape for the new leaf size
      rc = ensure_capacity(c, n);
      if (rc == GSPH_OK)
        for (int q = 0; q < 9; q++) {
          const cudaError_t e = cudaMemcpyAsync(c->in[q], save + (size_t) q * n, sizeof(double) * n,
                                                cudaMemcpyDeviceToDevice, c->stream);
          if (e != cudaSuccess) { rc = cuda_fail(c, e, "restore particles"); break; }
        }
      cudaStreamSynchronize(c->stream);
      cudaFree(save);
      if (rc != GSPH_OK) { c->cfg.nleafmax = old; return rc; }
      c->have_particles = true;
    }
    drop_graph(c);
    drop_kdk_graph(c);
    c->kdk = false;
    c->have_tree = c->have_props = c->have_forces = false;
  }
  if (t->near_depth != c->near_depth || t->cell_depth != c->cell_depth || t->gather_depth != c->gather_depth) {
    drop_graph(c);       // the captured launches hold the parameters by value
    drop_kdk_graph(c);
  }
  c->near_depth = t->near_depth;
  c->cell_depth = t->cell_depth;
  c->gather_depth = t->gather_depth;
  return GSPH_OK;
}

int32_t gsph_autotune(gsph_ctx* c, int32_t steps, gsph_tuning* best, gsph_tuning* tried, double* ms,
                      int32_t max_tried, int32_t* ntried) {
  if (!c || !best) return GSPH_ERR_INVALID;
  if (!c->have_particles) return fail(c, GSPH_ERR_STATE, "no particles imported");
  if (c->bactive) return fail(c, GSPH_ERR_STATE, "tune on structure-of-arrays imports");
  if (steps < 1 || steps > 1000) return fail(c, GSPH_ERR_INVALID, "steps out of range");
  cudaSetDevice(c->device);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  GSPH_CUDA(cudaEventCreate(&e0));
  GSPH_CUDA(cudaEventCreate(&e1));
  int count = 0;
  auto time_one = [&](const gsph_tuning& t, double& out_ms) -> int {
    int rc = gsph_set_tuning(c, &t);
    if (rc) return rc;
    rc = gsph_step_graph(c);   // capture and a first run, untimed
    if (rc) return rc;
    if (cudaEventRecord(e0, c->stream) != cudaSuccess) return cuda_fail(c, cudaGetLastError(), "event");
    for (int q = 0; q < steps && !rc; q++) rc = gsph_step_graph(c);
    if (rc) return rc;
    if (cudaEventRecord(e1, c->stream) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess)
      return cuda_fail(c, cudaGetLastError(), "event");
    float f = 0.0f;
    cudaEventElapsedTime(&f, e0, e1);
    out_ms = f / steps;
    if (tried && ms && count < max_tried) { tried[count] = t; ms[count] = out_ms; }
    count++;
    return GSPH_OK;
  };
  gsph_tuning cur{};
  gsph_get_tuning(c, &cur);
  gsph_tuning bestt = cur;
  double best_ms = 1e300;
  int rc = GSPH_OK;
  // leaf size with the current depths, then each depth in turn
  const int leaves[] = {4, 6, 8, 12, 16};
  for (int nl : leaves) {
    gsph_tuning t = bestt;
    t.nleafmax = nl;
    double m = 0.0;
    if (time_one(t, m) == GSPH_OK && m < best_ms) { best_ms = m; bestt = t; }
  }
  const bool mix = c->cfg.precision == GSPH_PRECISION_MIXED;
  if (mix && best_ms < 1e300) {
    const int nears[] = {64, 128, 256}, cells[] = {128, 256, 512}, gathers[] = {64, 128, 256};
    for (int v : nears) {
      gsph_tuning t = bestt;
      t.near_depth = v;
      double m = 0.0;
      if (time_one(t, m) == GSPH_OK && m < best_ms) { best_ms = m; bestt = t; }
    }
    for (int v : cells) {
      gsph_tuning t = bestt;
      t.cell_depth = v;
      double m = 0.0;
      if (time_one(t, m) == GSPH_OK && m < best_ms) { best_ms = m; bestt = t; }
    }
    for (int v : gathers) {
      gsph_tuning t = bestt;
      t.gather_depth = v;
      double m = 0.0;
      if (time_one(t, m) == GSPH_OK && m < best_ms) { best_ms = m; bestt = t; }
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (ntried) *ntried = count;
  if (best_ms >= 1e300) return fail(c, GSPH_ERR_STATE, "no candidate ran");
  rc = gsph_set_tuning(c, &bestt);
  if (rc) return rc;
  *best = bestt;
  return GSPH_OK;
}

}  // extern "C"

// ======================================================================================
// Batches of simulations (gsph_batch_*): one persistent launch per pass over the leaf
// cells of all simulations, the per-simulation tree builds and cell updates as parallel
// branches of one CUDA graph.
// ======================================================================================
struct gsph_batch {
  std::vector<gsph_ctx*> ctx;
  int device = 0;
  cudaStream_t stream = nullptr;
  SimDesc* d_sims = nullptr;
  int *d_start = nullptr, *d_hstart = nullptr, *d_next = nullptr;
  std::vector<int> key_n, key_cap, key_rec;
  std::vector<const void*> key_ptr;
  bool prepared = false, gravity = false;
  int lpg = 4;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaEvent_t fork[3] = {};
  std::vector<cudaEvent_t> join;   // 3 per simulation
  cudaEvent_t ev[2] = {};
  unsigned launches = 0;
  float ms = 0.0f;
  std::string err;
};

namespace {

int bfail(gsph_batch* b, int code, const std::string& msg) {
  b->err = msg;
  return code;
}

void batch_drop_graph(gsph_batch* b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->exec = nullptr;
  b->graph = nullptr;
}

bool batch_stale(const gsph_batch* b) {
  if (!b->prepared) return true;
  for (size_t i = 0; i < b->ctx.size(); i++) {
    const gsph_ctx* c = b->ctx[i];
    if (c->n != b->key_n[i] || c->cap != b->key_cap[i] || c->record != b->key_rec[i] ||
        (const void*) c->rec_sph_cnt != b->key_ptr[i])
      return true;
  }
  return false;
}

// Upload the simulations' descriptors and leaf prefix sums (host-synchronous).
int batch_prepare(gsph_batch* b) {
  const int ns = (int) b->ctx.size();
  std::vector<SimDesc> d(ns);
  std::vector<int> start(ns + 1, 0);
  b->lpg = 32;
  b->key_n.assign(ns, 0); b->key_cap.assign(ns, 0); b->key_rec.assign(ns, 0); b->key_ptr.assign(ns, nullptr);
  for (int i = 0; i < ns; i++) {
    gsph_ctx* c = b->ctx[i];
    if (!c->have_particles) return bfail(b, GSPH_ERR_STATE, "a simulation of the batch has no particles");
    if (c->nstar) return bfail(b, GSPH_ERR_UNSUPPORTED, "star particles are not supported in batches");
    int rc = ensure_recording(c);
    if (rc) return bfail(b, rc, c->err);
    d[i] = SimDesc{make_tree(c), make_particles(c), make_mixed_particles(c), make_mixed_cells(c), make_params(c),
                   make_counters(c), HeavyList{c->heavy_leaves, c->heavy_count}};
    start[i + 1] = start[i] + c->nleaf;
    b->lpg = std::min(b->lpg, c->lpg);
    b->key_n[i] = c->n; b->key_cap[i] = c->cap; b->key_rec[i] = c->record; b->key_ptr[i] = c->rec_sph_cnt;
  }
  cudaError_t e = cudaMemcpy(b->d_sims, d.data(), sizeof(SimDesc) * ns, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(b->d_start, start.data(), sizeof(int) * (ns + 1), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return bfail(b, GSPH_ERR_CUDA, std::string("batch upload: ") + cudaGetErrorString(e));
  batch_drop_graph(b);
  b->prepared = true;
  return GSPH_OK;
}

// The batch step in stream order (captured into the graph): per-simulation branches
// fork from and join the batch stream around each batched pass.
int batch_body(gsph_batch* b) {
  const int ns = (int) b->ctx.size();
  bool any_record = false;
  for (int i = 0; i < ns; i++) any_record = any_record || (b->ctx[i]->record && b->ctx[i]->rec_sph_cnt != nullptr);
  BatchQueue q{ns, b->d_sims, b->d_start, b->d_hstart, b->d_next, any_record};
  cudaStream_t o = b->stream;
  b->launches = 0;
  cudaEventRecordWithFlags(b->ev[0], o, cudaEventRecordExternal);
  auto branches = [&](int phase, auto&& work) -> int {
    cudaEventRecord(b->fork[phase], o);
    for (int i = 0; i < ns; i++) {
      gsph_ctx* c = b->ctx[i];
      c->stream = c->own_stream;
      cudaStreamWaitEvent(c->stream, b->fork[phase], 0);
      const int rc = work(c);
      if (rc) return bfail(b, rc, c->err);
      cudaEventRecord(b->join[3 * i + phase], c->stream);
      cudaStreamWaitEvent(o, b->join[3 * i + phase], 0);
    }
    return GSPH_OK;
  };
  int rc = branches(0, [&](gsph_ctx* c) -> int {
    int r = begin_counters(c);
    if (!r) r = do_build(c);
    if (!r && cudaMemsetAsync(c->heavy_count, 0, 4 * sizeof(int), c->stream) != cudaSuccess) r = GSPH_ERR_CUDA;
    return r;
  });
  if (rc) return rc;
  b->launches += (unsigned) launch_batch_density(q, b->lpg, o);
  rc = branches(1, [&](gsph_ctx* c) -> int {
    const Tree t = make_tree(c);
    const Particles p = make_particles(c);
    GSPH_CUDA(cudaMemcpyAsync(c->heavy_count + 2, c->heavy_count, sizeof(int), cudaMemcpyDeviceToDevice, c->stream));
    GSPH_CUDA(cudaMemsetAsync(c->heavy_count, 0, sizeof(int), c->stream));
    c->launches += (unsigned) launch_update_hmax(t, p, c->stream);
    launch_mixed_prep_hydro(t, p, make_mixed_particles(c), make_mixed_cells(c), c->stream);
    c->launches += 2;
    if (c->record && c->rec_sph_cnt) {
      GSPH_CUDA(cudaMemsetAsync(c->rec_sph_cnt, 0, sizeof(int) * (size_t) c->n, c->stream));
      GSPH_CUDA(cudaMemsetAsync(c->rec_dir_cnt, 0, sizeof(unsigned long long) * (size_t) c->n, c->stream));
      GSPH_CUDA(cudaMemsetAsync(c->rec_dir_hash, 0, sizeof(unsigned long long) * (size_t) c->n, c->stream));
      GSPH_CUDA(cudaMemsetAsync(c->rec_cell_cnt, 0, sizeof(unsigned long long) * (size_t) c->nleaf, c->stream));
      GSPH_CUDA(cudaMemsetAsync(c->rec_cell_hash, 0, sizeof(unsigned long long) * (size_t) c->nleaf, c->stream));
      if (c->rec_dir_max > 0 && c->rec_dir_n) {
        GSPH_CUDA(cudaMemsetAsync(c->rec_dir_n, 0, sizeof(int) * (size_t) c->n, c->stream));
        GSPH_CUDA(cudaMemsetAsync(c->rec_cell_n, 0, sizeof(int) * (size_t) c->nleaf, c->stream));
      }
    }
    return check_launch(c, "batch hmax update");
  });
  if (rc) return rc;
  b->launches += (unsigned) launch_batch_forces(q, b->gravity, b->lpg, o);
  rc = branches(2, [&](gsph_ctx* c) -> int {
    GSPH_CUDA(cudaMemcpyAsync(c->heavy_count + 3, c->heavy_count, sizeof(int), cudaMemcpyDeviceToDevice, c->stream));
    return GSPH_OK;
  });
  if (rc) return rc;
  cudaEventRecordWithFlags(b->ev[1], o, cudaEventRecordExternal);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return bfail(b, GSPH_ERR_CUDA, std::string("batch launch: ") + cudaGetErrorString(e));
  return GSPH_OK;
}

}  // namespace

extern "C" {

gsph_batch* gsph_batch_create(gsph_ctx* const* ctxs, int32_t nsim) {
  if (!ctxs || nsim < 1 || nsim > 4096) { g_create_error = GSPH_ERR_INVALID; return nullptr; }
  for (int i = 0; i < nsim; i++) {
    const gsph_ctx* c = ctxs[i];
    if (!c || c->device != ctxs[0]->device || c->cfg.precision != GSPH_PRECISION_MIXED ||
        c->cfg.self_gravity != ctxs[0]->cfg.self_gravity) {
      g_create_error = c && c->cfg.precision != GSPH_PRECISION_MIXED ? GSPH_ERR_UNSUPPORTED : GSPH_ERR_INVALID;
      return nullptr;
    }
    for (int j = 0; j < i; j++)
      if (ctxs[j] == c) { g_create_error = GSPH_ERR_INVALID; return nullptr; }
  }
  gsph_batch* b = new gsph_batch();
  b->ctx.assign(ctxs, ctxs + nsim);
  b->device = ctxs[0]->device;
  b->gravity = ctxs[0]->cfg.self_gravity != 0;
  cudaSetDevice(b->device);
  bool ok = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) == cudaSuccess;
  ok = ok && cudaMalloc(&b->d_sims, sizeof(SimDesc) * (size_t) nsim) == cudaSuccess;
  ok = ok && cudaMalloc(&b->d_start, sizeof(int) * (size_t) (nsim + 1)) == cudaSuccess;
  ok = ok && cudaMalloc(&b->d_hstart, sizeof(int) * (size_t) (nsim + 1)) == cudaSuccess;
  ok = ok && cudaMalloc(&b->d_next, sizeof(int) * 4) == cudaSuccess;
  for (int q = 0; q < 3 && ok; q++) ok = cudaEventCreateWithFlags(&b->fork[q], cudaEventDisableTiming) == cudaSuccess;
  b->join.assign(3 * (size_t) nsim, nullptr);
  for (auto& ev : b->join)
    if (ok) ok = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) == cudaSuccess;
  for (int q = 0; q < 2 && ok; q++) ok = cudaEventCreate(&b->ev[q]) == cudaSuccess;
  if (!ok) {
    gsph_batch_destroy(b);
    g_create_error = GSPH_ERR_CUDA;
    return nullptr;
  }
  g_create_error = GSPH_OK;
  return b;
}

void gsph_batch_destroy(gsph_batch* b) {
  if (!b) return;
  cudaSetDevice(b->device);
  if (b->stream) cudaStreamSynchronize(b->stream);
  batch_drop_graph(b);
  if (b->d_sims) cudaFree(b->d_sims);
  if (b->d_start) cudaFree(b->d_start);
  if (b->d_hstart) cudaFree(b->d_hstart);
  if (b->d_next) cudaFree(b->d_next);
  for (cudaEvent_t e : b->fork) if (e) cudaEventDestroy(e);
  for (cudaEvent_t e : b->join) if (e) cudaEventDestroy(e);
  for (cudaEvent_t e : b->ev) if (e) cudaEventDestroy(e);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
}

const char* gsph_batch_last_error(const gsph_batch* b) { return b ? b->err.c_str() : "null batch"; }

int32_t gsph_batch_step(gsph_batch* b) {
  if (!b) return GSPH_ERR_INVALID;
  cudaSetDevice(b->device);
  for (gsph_ctx* c : b->ctx) {
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) return bfail(b, GSPH_ERR_CUDA, "simulation stream");
  }
  int rc = GSPH_OK;
  if (batch_stale(b)) {
    rc = batch_prepare(b);
    if (rc) return rc;
  }
  std::vector<cudaStream_t> saved;
  for (gsph_ctx* c : b->ctx) saved.push_back(c->stream);
  if (!b->exec) {
    if (cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeRelaxed) != cudaSuccess)
      return bfail(b, GSPH_ERR_CUDA, "cudaStreamBeginCapture");
    for (gsph_ctx* c : b->ctx) c->capturing = true;
    rc = batch_body(b);
    for (gsph_ctx* c : b->ctx) c->capturing = false;
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(b->stream, &g);
    for (size_t i = 0; i < b->ctx.size(); i++) b->ctx[i]->stream = saved[i];
    if (rc) { if (g) cudaGraphDestroy(g); return rc; }
    if (e != cudaSuccess) return bfail(b, GSPH_ERR_CUDA, std::string("cudaStreamEndCapture: ") + cudaGetErrorString(e));
    b->graph = g;
    if (cudaGraphInstantiate(&b->exec, b->graph, 0) != cudaSuccess) {
      batch_drop_graph(b);
      return bfail(b, GSPH_ERR_CUDA, "cudaGraphInstantiate");
    }
  }
  if (cudaGraphLaunch(b->exec, b->stream) != cudaSuccess) return bfail(b, GSPH_ERR_CUDA, "cudaGraphLaunch");
  if (cudaStreamSynchronize(b->stream) != cudaSuccess) return bfail(b, GSPH_ERR_CUDA, "batch step");
  if (cudaEventElapsedTime(&b->ms, b->ev[0], b->ev[1]) != cudaSuccess) b->ms = 0.0f;
  (void) cudaGetLastError();
  int first = GSPH_OK;
  for (gsph_ctx* c : b->ctx) {
    c->have_tree = c->have_props = c->have_forces = true;
    c->have_star_forces = false;
    const int r = read_status(c);
    c->last.ms_build = c->last.ms_density = c->last.ms_hmax = c->last.ms_forces = 0.0f;
    c->last.ms_total = 0.0f;
    if (r && !first) {
      first = r;
      b->err = c->err;
    }
  }
  return first;
}

int32_t gsph_batch_stats(const gsph_batch* b, float* ms, int32_t* launches) {
  if (!b) return GSPH_ERR_INVALID;
  unsigned total = b->launches;
  for (const gsph_ctx* c : b->ctx) total += c->launches;
  if (ms) *ms = b->ms;
  if (launches) *launches = (int32_t) total;
  return GSPH_OK;
}

}  // extern "C"

// ======================================================================================
// KDK leapfrog with block timesteps (gsph_kdk_*): SphSimulation::PostInitialConditionsSetup
// and MainLoop (src/Hydrodynamics/SphSimulation.cpp:203-565, :573-880) for the gas, on the
// device.
// ======================================================================================
namespace {

// keep[] order of integrate.cuh: the leaf-order fields they mirror
const int kKeepField[kKeep] = {kFRho, kFInvOmega, kFZeta, kFHfactor, kFHrangesqd, kFPressure, kFSound,
                               kFAX, kFAY, kFAZ, kFAGX, kFAGY, kFAGZ, kFGpot, kFDudt, kFDivV, kFGpotHydro};

void kdk_free(gsph_ctx* c) {
  drop_kdk_graph(c);
  for (cudaEvent_t e : c->pev) cudaEventDestroy(e);   // after the graph that records them
  c->pev.clear();
  c->pkind.clear();
  c->pused = 0;
  for (void* q : {(void*) c->kg, (void*) c->kdk_buf, (void*) c->kdk_ibuf, (void*) c->kdk_flags,
                  (void*) c->leaf_active, (void*) c->leaf_level, (void*) c->leaf_lvn})
    if (q) cudaFree(q);
  c->kg = nullptr; c->kdk_buf = nullptr; c->kdk_ibuf = nullptr; c->kdk_flags = nullptr;
  c->leaf_active = nullptr; c->leaf_level = nullptr; c->leaf_lvn = nullptr;
  c->kdk_cap = 0;
  c->kdk = false;
}

// Block-timestep state buffers (integration state, keep[] fields, flags, levels) for the
// current capacity; shared by the KDK integration and the record imports with flags.
int ensure_kdk_buffers(gsph_ctx* c) {
  if (c->kdk_cap >= c->cap && c->kg) return GSPH_OK;
  kdk_free(c);
  const size_t k2 = (size_t) c->cap;
  GSPH_CUDA(cudaMalloc(&c->kg, sizeof(KdkGlobal)));
  GSPH_CUDA(cudaMemsetAsync(c->kg, 0, sizeof(KdkGlobal), c->stream));
  GSPH_CUDA(cudaMalloc(&c->kdk_buf, sizeof(double) * (14 + kKeep) * k2));
  GSPH_CUDA(cudaMalloc(&c->kdk_ibuf, sizeof(int) * 5 * k2));
  GSPH_CUDA(cudaMalloc(&c->kdk_flags, k2));
  GSPH_CUDA(cudaMalloc(&c->leaf_active, k2));
  GSPH_CUDA(cudaMalloc(&c->leaf_level, sizeof(int) * k2));
  GSPH_CUDA(cudaMalloc(&c->leaf_lvn, sizeof(int) * k2));
  c->kdk_cap = c->cap;
  return GSPH_OK;
}

// The input-order array of the KDK state that holds a leaf-order field (nullptr: none).
const double* kdk_field_source(gsph_ctx* c, int leaf_field) {
  const KdkState s = make_kdk_state(c);
  if (leaf_field == kFH) return s.h;
  if (leaf_field == kFU) return s.u;
  for (int q = 0; q < kKeep; q++)
    if (kKeepField[q] == leaf_field) return s.keep[q];
  return nullptr;
}

KdkState make_kdk_state(gsph_ctx* c) {
  KdkState s{};
  const size_t k = (size_t) c->kdk_cap;
  s.n = c->n;
  s.x = c->in[0]; s.y = c->in[1]; s.z = c->in[2]; s.vx = c->in[3]; s.vy = c->in[4]; s.vz = c->in[5];
  s.u = c->in[7]; s.h = c->in[8];
  double* b = c->kdk_buf;
  for (int q = 0; q < 3; q++) { s.r0[q] = b + q * k; s.v0[q] = b + (3 + q) * k; s.a0[q] = b + (6 + q) * k; }
  s.u0 = b + 9 * k; s.dudt0 = b + 10 * k; s.dt = b + 11 * k; s.dt_next = b + 12 * k; s.tlast = b + 13 * k;
  for (int q = 0; q < kKeep; q++) s.keep[q] = b + (14 + q) * k;
  int* ib = c->kdk_ibuf;
  s.nlast = ib; s.nstep = ib + k; s.level = ib + 2 * k; s.levelneib = ib + 3 * k; s.bt_list = ib + 4 * k;
  s.flags = c->kdk_flags;
  return s;
}

KdkLeaf make_kdk_leaf(gsph_ctx* c) {
  KdkLeaf l{};
  l.n = c->n;
  l.id = c->id;
  l.slot_of = c->slot_of;
  for (int q = 0; q < kKeep; q++) l.f[q] = c->f[kKeepField[q]];
  l.h = c->f[kFH];
  l.u = c->f[kFU];
  l.active = c->leaf_active;
  l.level = c->leaf_level;
  l.lvn = c->leaf_lvn;
  return l;
}

// One h solve + force pass over the active particles of the current tree.
int kdk_pass(gsph_ctx* c, bool forces) {
  const KdkState s = make_kdk_state(c);
  const KdkLeaf l = make_kdk_leaf(c);
  launch_kdk_gather(s, l, c->kg, c->stream);
  c->launches += 1;
  int rc = do_props(c);
  if (rc) return rc;
  if (forces) {
    rc = do_forces(c, c->cfg.self_gravity != 0);
    if (rc) return rc;
  }
  launch_kdk_scatter(s, l, c->stream);
  c->launches += 1;
  return check_launch(c, "kdk pass");
}

constexpr int kKdkPasses = 3;   // the first force pass and up to two CheckTimesteps repeats
enum { kPhBuild = 0, kPhDensity = 1, kPhForces = 2, kPhKinds = 3 };
constexpr int kPhEventsPerStep = 2 * (1 + 2 * kKdkPasses);

// One phase boundary: the next event of the pool, recorded on the context's stream.
void pmark(gsph_ctx* c, int kind) {
  if (!c->ptiming || c->pused >= c->pev.size()) return;
  cudaEvent_t e = c->pev[c->pused];
  c->pkind[c->pused] = kind;
  c->pused++;
  if (c->capturing) cudaEventRecordWithFlags(e, c->stream, cudaEventRecordExternal);
  else cudaEventRecord(e, c->stream);
}

// Events for nsteps steps of phase timing (created outside any capture).
int ensure_phase_events(gsph_ctx* c, int nsteps) {
  const size_t need = (size_t) kPhEventsPerStep * (size_t) nsteps;
  while (c->pev.size() < need) {
    cudaEvent_t e = nullptr;
    GSPH_CUDA(cudaEventCreate(&e));
    c->pev.push_back(e);
  }
  c->pkind.assign(c->pev.size(), -1);
  c->pused = 0;
  return GSPH_OK;
}

// Device time of each phase kind over the recorded pairs (after the stream has finished).
void sum_phases(gsph_ctx* c, double* ms) {
  for (int k = 0; k < kPhKinds; k++) ms[k] = 0.0;
  for (size_t q = 0; q + 1 < c->pused; q += 2) {
    float t = 0.0f;
    if (c->pkind[q] >= 0 && cudaEventElapsedTime(&t, c->pev[q], c->pev[q + 1]) == cudaSuccess) ms[c->pkind[q]] += t;
  }
  (void) cudaGetLastError();
}

// The interaction counters (density, hydro, direct, cell pairs) copied to a snapshot slot.
__global__ void k_snap_counters(const unsigned long long* counters, unsigned long long* dst) {
  if (threadIdx.x < 4 && blockIdx.x == 0) dst[threadIdx.x] = counters[1 + threadIdx.x];
}

// Opens the conditional graph node of a CheckTimesteps repeat pass on the capturing stream:
// a kernel sets the condition from the count of particles the last check activated, and
// the pass is captured into the node's body on a stream of its own (nested for the third
// pass), so that the graph skips a pass that would find no active particle.
int cond_begin(gsph_ctx* c, int depth) {
  cudaStreamCaptureStatus st;
  cudaGraph_t g = nullptr;
  const cudaGraphNode_t* deps = nullptr;
  size_t nd = 0;
  GSPH_CUDA(cudaStreamGetCaptureInfo(c->stream, &st, nullptr, &g, &deps, nullptr, &nd));
  cudaGraphConditionalHandle h;
  GSPH_CUDA(cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault));
  launch_kdk_set_cond(h, c->kg, c->stream);
  c->launches += 1;
  GSPH_CUDA(cudaStreamGetCaptureInfo(c->stream, &st, nullptr, &g, &deps, nullptr, &nd));
  cudaGraphNodeParams p = {};
  p.type = cudaGraphNodeTypeConditional;
  p.conditional.handle = h;
  p.conditional.type = cudaGraphCondTypeIf;
  p.conditional.size = 1;
  cudaGraphNode_t node;
  GSPH_CUDA(cudaGraphAddNode(&node, g, deps, nullptr, nd, &p));
  GSPH_CUDA(cudaStreamUpdateCaptureDependencies(c->stream, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
  GSPH_CUDA(cudaStreamBeginCaptureToGraph(c->cond_stream[depth], p.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                          cudaStreamCaptureModeRelaxed));
  c->cond_saved[depth] = c->stream;
  c->stream = c->cond_stream[depth];
  c->in_body = depth + 1;
  return GSPH_OK;
}

int cond_end(gsph_ctx* c, int depth) {
  cudaGraph_t b = nullptr;
  const cudaError_t e = cudaStreamEndCapture(c->stream, &b);
  c->stream = c->cond_saved[depth];
  c->in_body = depth;
  if (e != cudaSuccess) return cuda_fail(c, e, "conditional body capture");
  return GSPH_OK;
}

// Stream launches only: whether the last CheckTimesteps activated particles (a host read).
int host_activecount(gsph_ctx* c, int& count) {
  KdkGlobal g{};
  GSPH_CUDA(cudaMemcpyAsync(&g, c->kg, sizeof(g), cudaMemcpyDeviceToHost, c->stream));
  GSPH_CUDA(cudaStreamSynchronize(c->stream));
  count = g.activecount;
  return GSPH_OK;
}

// One main-loop step.  step: index inside the current gsph_kdk_steps call (snapshot slots).
int kdk_step_body(gsph_ctx* c, int step) {
  const KdkState s = make_kdk_state(c);
  const KdkLeaf l = make_kdk_leaf(c);
  launch_kdk_begin(c->kg, c->stream);
  launch_kdk_advance(s, c->kp, c->kg, c->stream);
  c->launches += 2;
  pmark(c, kPhBuild);
  int rc = do_build(c);
  if (rc) return rc;
  pmark(c, kPhBuild);
  int opened = 0;
  for (int pass = 0; pass < kKdkPasses; pass++) {
    if (pass > 0) {
      // a repeat pass runs only when CheckTimesteps activated particles: a conditional
      // node in a captured graph, a host read otherwise (an empty pass changes nothing)
      if (c->capturing) {
        rc = cond_begin(c, pass - 1);
        if (rc) break;
        opened = pass;
      } else {
        int cnt = 0;
        rc = host_activecount(c, cnt);
        if (rc || cnt == 0) break;
      }
    }
    const unsigned before = c->launches;
    // the tree is the same for all passes of a step: the first gathers every persistent
    // field into leaf order, the later ones only refresh the active flags and levels
    if (pass == 0) launch_kdk_gather(s, l, c->kg, c->stream);
    else launch_kdk_refresh(s, l, c->kg, c->stream);
    c->launches += 1;
    const bool first = pass == 0 && c->kdk_snap && step < c->kdk_snap_steps;
    if (first) k_snap_counters<<<1, 32, 0, c->stream>>>(c->counters, c->kdk_snap + 8 * step);
    if (pass == 0) pmark(c, kPhDensity);
    rc = do_props(c);
    if (rc) break;
    if (pass == 0) { pmark(c, kPhDensity); pmark(c, kPhForces); }
    rc = do_forces(c, c->cfg.self_gravity != 0);
    if (rc) break;
    if (pass == 0) pmark(c, kPhForces);
    if (first) k_snap_counters<<<1, 32, 0, c->stream>>>(c->counters, c->kdk_snap + 8 * step + 4);
    launch_kdk_scatter_lvn(s, l, c->stream);
    launch_kdk_check(s, c->kp, c->kg, pass == kKdkPasses - 1, c->stream);
    c->launches += pass == kKdkPasses - 1 ? 4 : 3;
    if (pass > 0) c->kdk_cond_launches = c->launches - before;
  }
  // close the bodies, innermost first
  for (int d = opened; d > 0; d--) {
    const int r2 = cond_end(c, d - 1);
    if (!rc) rc = r2;
  }
  if (rc) return rc;
  launch_kdk_scatter_fields(s, l, c->stream);
  c->launches += 1;
  launch_kdk_timesteps(s, c->kp, c->kg, c->stream);
  launch_kdk_end(s, c->kp, c->kg, c->stream);
  c->launches += 6;
  return check_launch(c, "kdk step");
}

int kdk_read(gsph_ctx* c) {
  int rc = read_status(c);
  KdkGlobal g{};
  GSPH_CUDA(cudaMemcpy(&g, c->kg, sizeof(g), cudaMemcpyDeviceToHost));
  if (!rc && (g.status & kKdkTimestepInvalid)) rc = fail(c, GSPH_ERR_INVALID, "Hydro timestep too large or non-positive");
  if (!rc && (g.status & kKdkNotSettled))
    rc = fail(c, GSPH_ERR_CAPACITY, "neighbour timestep checks still activating particles after the last pass");
  return rc;
}

}  // namespace

extern "C" {

void gsph_kdk_config_defaults(gsph_kdk_config* k) {
  if (!k) return;
  std::memset(k, 0, sizeof(*k));
  k->nlevels = 1;            // Parameters.cpp:244-245, :239-240, :263
  k->level_diff_max = 1;
  k->courant_mult = 0.15;
  k->accel_mult = 0.3;
  k->energy_mult = 0.4;
}

int32_t gsph_kdk_setup(gsph_ctx* c, const gsph_kdk_config* k) {
  if (!c || !k) return GSPH_ERR_INVALID;
  if (!c->have_particles) return fail(c, GSPH_ERR_STATE, "no particles imported");
  if (k->nlevels < 1 || k->nlevels > 20 || k->level_diff_max < 1 || !(k->courant_mult > 0) ||
      !(k->accel_mult > 0) || !(k->energy_mult > 0))
    return fail(c, GSPH_ERR_INVALID, "bad KDK parameters");
  if (c->nstar) return fail(c, GSPH_ERR_UNSUPPORTED, "star particles need the N-body integrator (not implemented)");
  cudaSetDevice(c->device);
  GSPH_CUDA(cudaStreamSynchronize(c->stream));
  int rc0 = ensure_kdk_buffers(c);
  if (rc0) return rc0;
  drop_graph(c);   // the single-step graph was captured without the active flags
  c->bactive = false;
  KdkParams kp{};
  kp.nlevels = k->nlevels;
  kp.level_diff_max = k->level_diff_max;
  kp.energy_integration = c->cfg.eos == GSPH_EOS_ENERGY_EQN;
  kp.periodic = c->cfg.periodic;
  kp.courant_mult = k->courant_mult;
  kp.accel_mult = k->accel_mult;
  kp.energy_mult = k->energy_mult;
  for (int q = 0; q < 3; q++) {
    kp.boxmin[q] = c->cfg.boxmin[q];
    kp.boxmax[q] = c->cfg.boxmax[q];
    kp.boxsize[q] = c->cfg.boxmax[q] - c->cfg.boxmin[q];
  }
  // the K-step graph holds the parameters by value: a new set needs a new capture
  if (std::memcmp(&kp, &c->kp, sizeof(kp)) != 0) drop_kdk_graph(c);
  c->kp = kp;
  c->kdk = true;
  const KdkState s = make_kdk_state(c);
  int rc = begin_counters(c);
  if (rc) return rc;
  launch_kdk_setup_state(s, c->kg, c->stream);
  // h solve on the initial tree, then a new tree with the solved h, a second h solve and
  // the force pass (SphSimulation.cpp:305-466 with initial h provided)
  rc = do_build(c);
  if (!rc) rc = kdk_pass(c, false);
  if (!rc) rc = do_build(c);
  if (!rc) rc = kdk_pass(c, true);
  if (rc) { c->kdk = false; return rc; }
  launch_kdk_setup_finish(s, c->stream);
  launch_kdk_timesteps(s, c->kp, c->kg, c->stream);
  launch_kdk_end(s, c->kp, c->kg, c->stream);
  rc = check_launch(c, "kdk setup");
  if (rc) { c->kdk = false; return rc; }
  rc = kdk_read(c);
  if (rc) c->kdk = false;
  c->keep_current = rc == GSPH_OK;
  return rc;
}

int32_t gsph_kdk_steps(gsph_ctx* c, int32_t nsteps, int32_t use_graph) {
  if (!c) return GSPH_ERR_INVALID;
  if (!c->kdk) return fail(c, GSPH_ERR_STATE, "gsph_kdk_setup has not been run for these particles");
  if (c->nstar) return fail(c, GSPH_ERR_UNSUPPORTED, "star particles need the N-body integrator (not implemented)");
  if (nsteps < 1 || nsteps > 100000) return fail(c, GSPH_ERR_INVALID, "nsteps out of range");
  cudaSetDevice(c->device);
  for (int q = 0; q < 2; q++)
    if (!c->cond_stream[q]) GSPH_CUDA(cudaStreamCreateWithFlags(&c->cond_stream[q], cudaStreamNonBlocking));
  if (c->kdk_snap_steps < nsteps) {
    if (c->kdk_snap) cudaFree(c->kdk_snap);
    c->kdk_snap = nullptr;
    c->kdk_snap_steps = 0;
    drop_kdk_graph(c);   // a captured graph writes the old snapshot buffer
    GSPH_CUDA(cudaMalloc(&c->kdk_snap, sizeof(unsigned long long) * 8 * (size_t) nsteps));
    c->kdk_snap_steps = nsteps;
  }
  int rc = begin_counters(c);
  if (rc) return rc;
  mark(c, 0);
  if (!use_graph) {
    rc = ensure_phase_events(c, nsteps);
    if (rc) return rc;
    c->ptiming = true;
    for (int q = 0; q < nsteps && !rc; q++) rc = kdk_step_body(c, q);
    c->ptiming = false;
    if (rc) return rc;
  } else {
    if (!c->kdk_exec || c->kdk_graph_steps != nsteps) {
      if (c->kdk_exec) cudaGraphExecDestroy(c->kdk_exec);
      if (c->kdk_graph) cudaGraphDestroy(c->kdk_graph);
      c->kdk_exec = nullptr;
      c->kdk_graph = nullptr;
      GSPH_CUDA(cudaStreamSynchronize(c->stream));
      rc = ensure_phase_events(c, nsteps);   // the graph records these events on every replay
      if (rc) return rc;
      cudaStream_t saved = c->stream;
      c->stream = c->own_stream;
      const unsigned before = c->launches;
      GSPH_CUDA(cudaStreamBeginCapture(c->own_stream, cudaStreamCaptureModeRelaxed));
      c->capturing = true;
      c->ptiming = true;
      for (int q = 0; q < nsteps && !rc; q++) rc = kdk_step_body(c, q);
      c->ptiming = false;
      c->capturing = false;
      cudaGraph_t g = nullptr;
      const cudaError_t e = cudaStreamEndCapture(c->own_stream, &g);
      c->stream = saved;
      if (rc) { if (g) cudaGraphDestroy(g); return rc; }
      if (e != cudaSuccess) return cuda_fail(c, e, "cudaStreamEndCapture");
      c->kdk_graph = g;
      GSPH_CUDA(cudaGraphInstantiate(&c->kdk_exec, c->kdk_graph, 0));
      c->kdk_graph_steps = nsteps;
      c->kdk_graph_launches = c->launches - before;
    }
    // the counters were zeroed by begin_counters outside the graph
    GSPH_CUDA(cudaGraphLaunch(c->kdk_exec, c->stream));
    c->launches += c->kdk_graph_launches;
  }
  mark(c, 4);
  rc = kdk_read(c);
  float ms = 0.0f;
  if (cudaEventElapsedTime(&ms, c->ev[0], c->ev[4]) != cudaSuccess) ms = 0.0f;
  (void) cudaGetLastError();
  double ph[kPhKinds];
  sum_phases(c, ph);
  {
    gsph_kdk_timing& T = c->kdk_timing;
    T = gsph_kdk_timing{};
    T.ms_build = ph[kPhBuild];
    T.ms_density = ph[kPhDensity];
    T.ms_forces = ph[kPhForces];
    T.steps = nsteps;
    std::vector<unsigned long long> sn(8 * (size_t) nsteps);
    if (cudaMemcpy(sn.data(), c->kdk_snap, sizeof(unsigned long long) * sn.size(), cudaMemcpyDeviceToHost) ==
        cudaSuccess) {
      for (int q = 0; q < nsteps; q++) {
        const unsigned long long* a = &sn[8 * (size_t) q];
        T.density_pairs += (int64_t) (a[4] - a[0]);
        T.hydro_pairs += (int64_t) (a[5] - a[1]);
        T.direct_pairs += (int64_t) (a[6] - a[2]);
        T.cell_pairs += (int64_t) (a[7] - a[3]);
      }
    }
    KdkGlobal g{};
    if (cudaMemcpy(&g, c->kg, sizeof(g), cudaMemcpyDeviceToHost) == cudaSuccess) T.repeat_passes = (int64_t) g.repeat_passes;
    (void) cudaGetLastError();
  }
  // summed over the steps; the h solve phase includes the hmax update, the thermal update
  // and the mixed form's mirror refresh that follow it
  c->last.ms_build = ph[kPhBuild];
  c->last.ms_density = ph[kPhDensity];
  c->last.ms_hmax = 0.0;
  c->last.ms_forces = ph[kPhForces];
  c->last.ms_total = ms;
  c->have_tree = c->have_props = c->have_forces = true;
  c->keep_current = rc == GSPH_OK;
  return rc;
}

int32_t gsph_kdk_get_timing(gsph_ctx* c, gsph_kdk_timing* out) {
  if (!c || !out) return GSPH_ERR_INVALID;
  *out = c->kdk_timing;
  return GSPH_OK;
}

int32_t gsph_kdk_get_status(gsph_ctx* c, gsph_kdk_status* out) {
  if (!c || !out) return GSPH_ERR_INVALID;
  if (!c->kdk) return fail(c, GSPH_ERR_STATE, "no KDK integration in this context");
  cudaSetDevice(c->device);
  GSPH_CUDA(cudaStreamSynchronize(c->stream));
  KdkGlobal g{};
  GSPH_CUDA(cudaMemcpy(&g, c->kg, sizeof(g), cudaMemcpyDeviceToHost));
  out->n = g.n; out->nresync = g.nresync; out->level_max = g.level_max; out->level_step = g.level_step;
  out->nsteps = g.Nsteps; out->t = g.t; out->timestep = g.timestep; out->dt_max = g.dt_max;
  out->active_updates = (int64_t) g.active_updates;
  out->status = g.status;
  return GSPH_OK;
}

int32_t gsph_kdk_get_state(gsph_ctx* c, int32_t which, double* out) {
  if (!c || !out) return GSPH_ERR_INVALID;
  if (!c->kdk) return fail(c, GSPH_ERR_STATE, "no KDK integration in this context");
  if (which < 0 || which >= GSPH_KDK_COUNT) return fail(c, GSPH_ERR_INVALID, "unknown KDK state field");
  cudaSetDevice(c->device);
  GSPH_CUDA(cudaStreamSynchronize(c->stream));
  const KdkState s = make_kdk_state(c);
  const size_t n = (size_t) c->n;
  const double* src = nullptr;
  const int* isrc = nullptr;
  switch (which) {
    case GSPH_KDK_X: src = s.x; break;
    case GSPH_KDK_Y: src = s.y; break;
    case GSPH_KDK_Z: src = s.z; break;
    case GSPH_KDK_VX: src = s.vx; break;
    case GSPH_KDK_VY: src = s.vy; break;
    case GSPH_KDK_VZ: src = s.vz; break;
    case GSPH_KDK_U: src = s.u; break;
    case GSPH_KDK_DT: src = s.dt; break;
    case GSPH_KDK_TLAST: src = s.tlast; break;
    case GSPH_KDK_LEVEL: isrc = s.level; break;
    case GSPH_KDK_NSTEP: isrc = s.nstep; break;
    case GSPH_KDK_NLAST: isrc = s.nlast; break;
    default: isrc = s.levelneib; break;
  }
  if (src) {
    GSPH_CUDA(cudaMemcpy(out, src, sizeof(double) * n, cudaMemcpyDeviceToHost));
  } else {
    std::vector<int> v(n);
    GSPH_CUDA(cudaMemcpy(v.data(), isrc, sizeof(int) * n, cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < n; i++) out[i] = (double) v[i];
  }
  return GSPH_OK;
}

}  // extern "C"
