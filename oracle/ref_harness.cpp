// Test infrastructure only: drives the upstream GANDALF library (compiled from its own
// sources by oracle/Makefile.ref) through one particle step and dumps what it computed.
//
// The step is the one a steady-state SphSimulation::MainLoop performs for the hot path
// (src/Hydrodynamics/SphSimulation.cpp:634-757):
//   HydroTree::BuildTree (rebuild)            src/Tree/HydroTree.cpp:309-372
//   SearchBoundaryGhostParticles/BuildGhostTree  src/Tree/HydroTree.cpp:381-543
//   GradhSphTree::UpdateAllSphProperties       src/GradhSph/GradhSphTree.cpp:82-271
//   zero accelerations                         src/Hydrodynamics/SphSimulation.cpp:416-431
//   GradhSphTree::UpdateAllSphForces | UpdateAllSphHydroForces
//                                              src/GradhSph/GradhSphTree.cpp:279-657
//   HydroTree::UpdateAllStarGasForces (stars)  src/Tree/HydroTree.cpp:551-654
// and then re-runs the reference's own walks on the built tree to extract neighbour and
// gravity interaction lists (src/Tree/Tree.cpp:561-735, src/Headers/NeighbourManager.h).
//
// usage: gsph_ref_harness <input.bin> <outdir>
//   input.bin  : written by oracle/refio.py (header + SoA particle arrays, input order,
//                then, when the header's nstar > 0, the star arrays x y z vx vy vz m h)
//   outdir     : receives particles.bin, cells.bin, leaves.bin, lists.bin, timing.txt
//                and, with stars, stars.bin (a[3] adot[3] gpot per star)
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cstdint>
#include <chrono>
#include <string>
#include <vector>
#include <unistd.h>

#include "Precision.h"
#include "Exception.h"
#include "Parameters.h"
#include "Simulation.h"
#include "SphNeighbourSearch.h"
#include "NeighbourManager.h"
#include "KDTree.h"

namespace {

struct InHeader {
  char magic[8];          // "GSPHIN01"
  int32_t n;
  int32_t self_gravity;
  int32_t eos;            // 0 energy_eqn (adiabatic), 1 isothermal
  int32_t periodic;       // 0 open, 1 periodic in x,y,z
  int32_t nleafmax;
  int32_t multipole;      // 0 monopole, 1 quadrupole
  int32_t nstar;          // star particles following the gas arrays
  int32_t kdk;            // 1: a KdkBlock follows the header (multi-step run)
  double h_fac, h_converge, alpha_visc, beta_visc, gamma_eos, thetamaxsqd, temp0, mu_bar;
  double boxmin[3], boxmax[3];
};

// Multi-step run: SetupSimulation then nsteps SphSimulation::MainLoop calls
// (src/Hydrodynamics/SphSimulation.cpp:573-880) with the KDK leapfrog and block timesteps.
struct KdkBlock {
  int32_t nsteps, nlevels, level_diff_max, pad;
  double courant_mult, accel_mult, energy_mult, pad2;
};

void die(const char* msg) { std::fprintf(stderr, "gsph_ref_harness: %s\n", msg); std::exit(2); }

template <typename T>
void write_block(FILE* f, const std::vector<T>& v) {
  int64_t n = (int64_t) v.size();
  std::fwrite(&n, sizeof(n), 1, f);
  if (n) std::fwrite(v.data(), sizeof(T), v.size(), f);
}

double now_s() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

}  // namespace

int main(int argc, char** argv) {
  if (argc != 3) die("usage: gsph_ref_harness <input.bin> <outdir>");
  const std::string outdir = argv[2];

  FILE* fin = std::fopen(argv[1], "rb");
  if (!fin) die("cannot open input");
  InHeader hd;
  if (std::fread(&hd, sizeof(hd), 1, fin) != 1) die("short header");
  if (std::memcmp(hd.magic, "GSPHIN01", 8) != 0) die("bad magic");
  KdkBlock kb{};
  if (hd.kdk && std::fread(&kb, sizeof(kb), 1, fin) != 1) die("short kdk block");
  const int N = hd.n;
  std::vector<double> arr[9];
  for (int a = 0; a < 9; a++) {
    arr[a].resize(N);
    if (std::fread(arr[a].data(), sizeof(double), N, fin) != (size_t) N) die("short array");
  }
  const int NS = hd.nstar;
  std::vector<double> sarr[8];
  for (int a = 0; a < 8 && NS > 0; a++) {
    sarr[a].resize(NS);
    if (std::fread(sarr[a].data(), sizeof(double), NS, fin) != (size_t) NS) die("short star array");
  }
  std::fclose(fin);
  // x y z vx vy vz m u h
  std::vector<double>& h_in = arr[8];

  // The reference writes snapshot/param files into the working directory.
  if (chdir(outdir.c_str()) != 0) die("cannot chdir to outdir");

  ExceptionHandler::makeExceptionHandler(cplusplus);
  Parameters* params = new Parameters();
  auto S = [&](const char* k, const std::string& v) { params->stringparams[k] = v; };
  auto I = [&](const char* k, int v) { params->intparams[k] = v; };
  auto F = [&](const char* k, double v) { params->floatparams[k] = v; };
  S("ic", "python"); S("sim", "sph"); S("run_id", "refrun"); S("out_file_form", "column");
  I("ndim", 3); I("Nhydro", N); I("Nstar", NS); I("dimensionless", 1);
  S("kernel", "m4"); I("tabulated_kernel", 0);
  F("h_fac", hd.h_fac); F("h_converge", hd.h_converge);
  S("avisc", "mon97"); S("acond", "none"); S("time_dependent_avisc", "none");
  F("alpha_visc", hd.alpha_visc); F("beta_visc", hd.beta_visc);
  S("gas_eos", hd.eos == 1 ? "isothermal" : "energy_eqn");
  F("gamma_eos", hd.gamma_eos); F("temp0", hd.temp0); F("mu_bar", hd.mu_bar);
  I("hydro_forces", 1); I("self_gravity", hd.self_gravity);
  S("neib_search", "kdtree"); S("gravity_mac", "geometric");
  S("multipole", hd.multipole == 1 ? "quadrupole" : "monopole");
  I("Nleafmax", hd.nleafmax); F("thetamaxsqd", hd.thetamaxsqd);
  I("ntreebuildstep", 1); I("ntreestockstep", 1);
  I("Nlevels", hd.kdk ? kb.nlevels : 1); I("sink_particles", 0);
  if (hd.kdk) {
    I("level_diff_max", kb.level_diff_max);
    F("courant_mult", kb.courant_mult); F("accel_mult", kb.accel_mult); F("energy_mult", kb.energy_mult);
  }
  S("sph_integration", "lfkdk");
  const char* bl[3] = {"boundary_lhs[0]", "boundary_lhs[1]", "boundary_lhs[2]"};
  const char* br[3] = {"boundary_rhs[0]", "boundary_rhs[1]", "boundary_rhs[2]"};
  const char* bmn[3] = {"boxmin[0]", "boxmin[1]", "boxmin[2]"};
  const char* bmx[3] = {"boxmax[0]", "boxmax[1]", "boxmax[2]"};
  for (int k = 0; k < 3; k++) {
    S(bl[k], hd.periodic ? "periodic" : "open");
    S(br[k], hd.periodic ? "periodic" : "open");
    if (hd.periodic) { F(bmn[k], hd.boxmin[k]); F(bmx[k], hd.boxmax[k]); }
  }

  SimulationBase* base = SimulationBase::SimulationFactory(3, "sph", params);
  base->PreSetupForPython();
  const char* names[9] = {"x", "y", "z", "vx", "vy", "vz", "m", "u", "h"};
  for (int a = 0; a < 9; a++) base->ImportArray(arr[a].data(), N, names[a]);
  const char* snames[8] = {"x", "y", "z", "vx", "vy", "vz", "m", "h"};
  for (int a = 0; a < 8 && NS > 0; a++) base->ImportArray(sarr[a].data(), NS, snames[a], "star");
  // Never initialised on the Python path (Simulation.h:163); the inputs carry h.
  base->initial_h_provided = true;
  const double t_setup0 = now_s();
  base->SetupSimulation();
  const double t_setup = now_s() - t_setup0;

  GradhSphSimulation<3>* sim = static_cast<GradhSphSimulation<3>*>(base);
  if (hd.kdk) {
    // ---- multi-step run: the reference's own main loop ----------------------------------
    const double tk0 = now_s();
    for (int s = 0; s < kb.nsteps; s++) sim->MainLoop();
    const double tk = now_s() - tk0;
    Sph<3>* sp = sim->sph;
    const int NK = 24;
    std::vector<double> kout((size_t) N * NK);
    for (int i = 0; i < N; i++) {
      GradhSphParticle<3>& p = static_cast<GradhSphParticle<3>&>(sp->GetSphParticlePointer(i));
      if (p.iorig != i) die("particle order changed");
      double* o = &kout[(size_t) i * NK];
      for (int k = 0; k < 3; k++) { o[k] = p.r[k]; o[3 + k] = p.v[k]; o[6 + k] = p.a[k]; }
      o[9] = p.h; o[10] = p.rho; o[11] = p.u; o[12] = p.level; o[13] = p.nstep; o[14] = p.nlast;
      o[15] = p.levelneib; o[16] = p.dt; o[17] = p.tlast; o[18] = p.dudt; o[19] = p.div_v;
      o[20] = p.gpot; o[21] = p.invomega; o[22] = p.pressure; o[23] = p.sound;
    }
    std::vector<double> g = {(double) sim->n, sim->t, sim->timestep, (double) sim->level_max,
                             (double) sim->level_step, (double) sim->nresync, (double) sim->Nsteps, sim->dt_max};
    FILE* fk = std::fopen("kdk.bin", "wb");
    write_block(fk, kout);
    write_block(fk, g);
    std::fclose(fk);
    fk = std::fopen("timing.txt", "w");
    std::fprintf(fk, "setup %.6f\nkdk_steps %.6f\n", t_setup, tk);
    std::fclose(fk);
    return 0;
  }
  Sph<3>* sph = sim->sph;
  typedef GradhSphTree<3, GradhSphParticle> TreeType;
  TreeType* neib = reinterpret_cast<TreeType*>(sim->sphneib);
  typedef KDTree<3, GradhSphParticle, KDTreeCell> KD;
  KD* tree = static_cast<KD*>(neib->tree);

  // ---- the controlled step: restart from the input smoothing lengths -------------------
  for (int i = 0; i < sph->Nhydro; i++) {
    GradhSphParticle<3>& p = static_cast<GradhSphParticle<3>&>(sph->GetSphParticlePointer(i));
    p.h = h_in[i];
    p.flags.set(active);
  }
  const double t0 = now_s();
  neib->BuildTree(true, 0, 1, 1, (FLOAT) 0.0, sph);
  const double t1 = now_s();
  neib->SearchBoundaryGhostParticles((FLOAT) 0.0, sim->simbox, sph);
  neib->BuildGhostTree(true, 0, 1, 1, (FLOAT) 0.0, sph);
  const double t2 = now_s();
  neib->UpdateAllSphProperties(sph, sim->nbody);
  const double t3 = now_s();
  for (int i = 0; i < sph->Nhydro; i++) {
    GradhSphParticle<3>& p = static_cast<GradhSphParticle<3>&>(sph->GetSphParticlePointer(i));
    p.levelneib = 0; p.dalphadt = 0; p.div_v = 0; p.dudt = 0; p.gpot = 0; p.gpot_hydro = 0;
    for (int k = 0; k < 3; k++) { p.a[k] = 0; p.atree[k] = 0; }
  }
  if (hd.self_gravity) neib->UpdateAllSphForces(sph, sim->nbody, sim->simbox, sim->ewald);
  else neib->UpdateAllSphHydroForces(sph, sim->nbody, sim->simbox);
  const double t4 = now_s();

  // ---- star <- gas forces (HydroTree::UpdateAllStarGasForces) --------------------------
  std::vector<double> sout((size_t) NS * 7);
  if (NS > 0) {
    Nbody<3>* nb = sim->nbody;
    for (int s = 0; s < nb->Nnbody; s++) {
      NbodyParticle<3>* st = nb->nbodydata[s];
      for (int k = 0; k < 3; k++) { st->a[k] = 0; st->adot[k] = 0; }
      st->gpot = 0;
      st->flags.set(active);
    }
    if (hd.self_gravity) neib->UpdateAllStarGasForces(sph, nb, sim->simbox, sim->ewald);
    for (int s = 0; s < NS; s++) {
      NbodyParticle<3>* st = nb->nbodydata[s];
      double* o = &sout[(size_t) s * 7];
      for (int k = 0; k < 3; k++) { o[k] = st->a[k]; o[3 + k] = st->adot[k]; }
      o[6] = st->gpot;
    }
  }

  // ---- per-particle results (input order) --------------------------------------------
  const int NP = 20;
  std::vector<double> pout((size_t) N * NP);
  for (int i = 0; i < N; i++) {
    GradhSphParticle<3>& p = static_cast<GradhSphParticle<3>&>(sph->GetSphParticlePointer(i));
    if (p.iorig != i) die("particle order changed");
    double* o = &pout[(size_t) i * NP];
    o[0] = p.h; o[1] = p.rho; o[2] = p.invomega; o[3] = p.zeta; o[4] = p.hfactor;
    o[5] = p.pressure; o[6] = p.sound; o[7] = p.u; o[8] = p.div_v; o[9] = p.dudt;
    o[10] = p.a[0]; o[11] = p.a[1]; o[12] = p.a[2];
    o[13] = p.atree[0]; o[14] = p.atree[1]; o[15] = p.atree[2];
    o[16] = p.gpot; o[17] = p.gpot_hydro; o[18] = p.hrangesqd; o[19] = (double) p.levelneib;
  }

  // ---- tree cells (DFS order) and leaf particle sets --------------------------------
  const int NC = 34;
  std::vector<double> cout_((size_t) tree->Ncell * NC);
  std::vector<int32_t> leafpart;       // concatenated leaf member ids
  std::vector<int32_t> leafoff(1, 0);  // per leaf (in DFS order) offsets
  std::vector<int32_t> leafcell;       // DFS id of each leaf
  for (int c = 0; c < tree->Ncell; c++) {
    const KDTreeCell<3>& cell = tree->celldata[c];
    double* o = &cout_[(size_t) c * NC];
    o[0] = cell.N; o[1] = cell.level; o[2] = cell.copen; o[3] = cell.cnext;
    for (int k = 0; k < 3; k++) { o[4 + k] = cell.bb.min[k]; o[7 + k] = cell.bb.max[k]; }
    for (int k = 0; k < 3; k++) { o[10 + k] = cell.hbox.min[k]; o[13 + k] = cell.hbox.max[k]; }
    for (int k = 0; k < 3; k++) { o[16 + k] = cell.rcell[k]; o[19 + k] = cell.r[k]; }
    o[22] = cell.m; o[23] = cell.rmax; o[24] = cell.hmax; o[25] = cell.cdistsqd;
    for (int k = 0; k < 5; k++) o[26 + k] = cell.q[k];
    o[31] = cell.maxsound; o[32] = cell.Nactive; o[33] = cell.id;
    if (cell.copen == -1) {
      leafcell.push_back(c);
      int i = cell.ifirst;
      while (i != -1) {
        leafpart.push_back(i);
        if (i == cell.ilast) break;
        i = tree->inext[i];
      }
      leafoff.push_back((int32_t) leafpart.size());
    }
  }

  // ---- neighbour / interaction lists from the reference's own walks -----------------
  // hydro (SPH) neighbour lists per particle (input order), CSR
  std::vector<int32_t> nh_off(N + 1, 0), nh_ids;
  std::vector<std::vector<int32_t>> nh(N), gdir(N), gsm(N);
  std::vector<int32_t> gcell_off(1, 0), gcell_ids, gcell_leaf;
  {
    vector<TreeCellBase<3> > celllist;
    const int cactive = tree->ComputeActiveCellList(celllist);
    typedef GradhSphParticle<3>::HydroForcesParticle HP;
    NeighbourManager<3, HP> nm(sph, sim->simbox);
    GradhSphParticle<3>* sphdata = static_cast<GradhSphParticle<3>*>(sph->GetSphParticleArray());
    std::vector<int> activelist(tree->MaxNumPartInLeafCell() + 8);
    for (int cc = 0; cc < cactive; cc++) {
      TreeCellBase<3>& cell = celllist[cc];
      const int Nactive = tree->ComputeActiveParticleList(cell, sphdata, activelist.data());
      nm.clear();
      if (hd.self_gravity) {
        tree->ComputeGravityInteractionAndGhostList(cell, nm);
        nm.EndSearchGravity(cell, sphdata);
        MultipoleMoment<3>* gravcell;
        const int Ng = nm.GetGravCell(&gravcell);
        gcell_leaf.push_back(cell.id);
        for (int g = 0; g < Ng; g++) gcell_ids.push_back(gravcell[g].id);
        gcell_off.push_back((int32_t) gcell_ids.size());
      } else {
        tree->ComputeNeighbourAndGhostList(cell, nm);
        nm.EndSearch(cell, sphdata);
      }
      for (int j = 0; j < Nactive; j++) {
        const int i = activelist[j];
        GradhSphParticle<3>& p = sphdata[i];
        Typemask hydromask = sph->types[p.ptype].hydromask;
        if (hd.self_gravity) {
          GravityNeighbourLists<HP> lists = nm.GetParticleNeibGravity(p, hydromask);
          for (size_t q = 0; q < lists.neiblist.size(); q++) nh[i].push_back(lists.neiblist[q].iorig);
          for (size_t q = 0; q < lists.directlist.size(); q++) gdir[i].push_back(lists.directlist[q].iorig);
          for (size_t q = 0; q < lists.smooth_gravlist.size(); q++) gsm[i].push_back(lists.smooth_gravlist[q].iorig);
        } else {
          NeighbourList<HP> list = nm.GetParticleNeib(p, hydromask, false);
          for (size_t q = 0; q < list.size(); q++) nh[i].push_back(list[q].iorig);
        }
      }
    }
  }
  std::vector<int32_t> gd_off(N + 1, 0), gd_ids, gs_off(N + 1, 0), gs_ids;
  for (int i = 0; i < N; i++) {
    nh_ids.insert(nh_ids.end(), nh[i].begin(), nh[i].end()); nh_off[i + 1] = (int32_t) nh_ids.size();
    gd_ids.insert(gd_ids.end(), gdir[i].begin(), gdir[i].end()); gd_off[i + 1] = (int32_t) gd_ids.size();
    gs_ids.insert(gs_ids.end(), gsm[i].begin(), gsm[i].end()); gs_off[i + 1] = (int32_t) gs_ids.size();
  }

  FILE* f = std::fopen("particles.bin", "wb"); write_block(f, pout); std::fclose(f);
  f = std::fopen("cells.bin", "wb"); write_block(f, cout_); std::fclose(f);
  f = std::fopen("leaves.bin", "wb");
  write_block(f, leafcell); write_block(f, leafoff); write_block(f, leafpart); std::fclose(f);
  f = std::fopen("lists.bin", "wb");
  write_block(f, nh_off); write_block(f, nh_ids);
  write_block(f, gd_off); write_block(f, gd_ids);
  write_block(f, gs_off); write_block(f, gs_ids);
  write_block(f, gcell_leaf); write_block(f, gcell_off); write_block(f, gcell_ids);
  std::fclose(f);
  if (NS > 0) { f = std::fopen("stars.bin", "wb"); write_block(f, sout); std::fclose(f); }
  f = std::fopen("timing.txt", "w");
  std::fprintf(f, "setup %.6f\nbuild_tree %.6f\nghosts %.6f\nsph_properties %.6f\nforces %.6f\n"
               "step_total %.6f\nltot %d\nncell %d\n",
               t_setup, t1 - t0, t2 - t1, t3 - t2, t4 - t3, t4 - t0, tree->ltot, tree->Ncell);
  std::fclose(f);
  return 0;
}
