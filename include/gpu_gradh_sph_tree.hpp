// gpu_gradh_sph_tree.hpp — the GANDALF-side drop-in for libgsph_gb300.
//
// A GradhSphTree<ndim,ParticleType> (src/Headers/SphNeighbourSearch.h:173-227) whose hot
// path runs through the C ABI of include/gsph_gb300.h.  A GANDALF maintainer adds this
// header to the GANDALF tree (it includes GANDALF's own headers) and constructs
// GpuGradhSphTree instead of GradhSphTree in GradhSphSimulation::ProcessSphParameters
// (src/GradhSph/GradhSphSimulation.cpp:243-246).  The host particle array stays the source
// of truth: every call reads the records it needs and writes back only the fields the
// reference writes, for the active particles only (block timesteps).
//
// ndim must be 3 and ParticleType GradhSphParticle (the library's path).
#ifndef GPU_GRADH_SPH_TREE_HPP_
#define GPU_GRADH_SPH_TREE_HPP_

#include <cstddef>
#include <string>

#include "SphNeighbourSearch.h"
#include "gsph_gb300.h"

template <int ndim, template <int> class ParticleType>
class GpuGradhSphTree : public GradhSphTree<ndim, ParticleType> {
 public:
  typedef ParticleType<ndim> P;

  GpuGradhSphTree(std::string tree_type, int Nleafmax, int Nmpi, int pruning_level_min, int pruning_level_max,
                  FLOAT thetamaxsqd, FLOAT kernrange, FLOAT macerror, std::string gravity_mac,
                  std::string multipole, DomainBox<ndim>* box, SmoothingKernel<ndim>* kern, CodeTiming* timing,
                  ParticleTypeRegister& types, const gsph_config& cfg, int device = 0)
      : GradhSphTree<ndim, ParticleType>(tree_type, Nleafmax, Nmpi, pruning_level_min, pruning_level_max,
                                         thetamaxsqd, kernrange, macerror, gravity_mac, multipole, box, kern,
                                         timing, types) {
    static_assert(ndim == 3, "libgsph_gb300 implements ndim = 3");
    ctx_ = gsph_create(&cfg, device);
    if (!ctx_) ExceptionHandler::getIstance().raise("gsph_create failed");
    off_.r = offsetof(P, r);                 off_.v = offsetof(P, v);
    off_.m = offsetof(P, m);                 off_.h = offsetof(P, h);
    off_.u = offsetof(P, u);                 off_.rho = offsetof(P, rho);
    off_.invomega = offsetof(P, invomega);   off_.zeta = offsetof(P, zeta);
    off_.hfactor = offsetof(P, hfactor);     off_.hrangesqd = offsetof(P, hrangesqd);
    off_.pressure = offsetof(P, pressure);   off_.sound = offsetof(P, sound);
    off_.div_v = offsetof(P, div_v);         off_.dudt = offsetof(P, dudt);
    off_.a = offsetof(P, a);                 off_.atree = offsetof(P, atree);
    off_.gpot = offsetof(P, gpot);           off_.gpot_hydro = offsetof(P, gpot_hydro);
    off_.flags = offsetof(P, flags);         off_.level = offsetof(P, level);
    off_.levelneib = offsetof(P, levelneib);
  }
  virtual ~GpuGradhSphTree() { gsph_destroy(ctx_); }

  // HydroTree::BuildTree (src/Tree/HydroTree.cpp:309-372): records in, tree built.  The
  // periodic ghosts the reference makes (BuildGhostTree, SearchBoundaryGhostParticles) are
  // formed on the GPU, so those two calls have nothing left to do.
  virtual void BuildTree(const bool, const int, const int, const int, const FLOAT, Hydrodynamics<ndim>* hydro) {
    check(gsph_set_particles_aos(ctx_, hydro->template GetParticleArray<ParticleType>(), hydro->Nhydro,
                                 sizeof(P), &off_));
    check(gsph_build_tree(ctx_));
  }
  virtual void BuildGhostTree(const bool, const int, const int, const int, const FLOAT, Hydrodynamics<ndim>*) {}
  virtual void SearchBoundaryGhostParticles(FLOAT, const DomainBox<ndim>&, Hydrodynamics<ndim>*) {}

  // KDTree::UpdateActiveParticleCounters via HydroTree (src/Tree/HydroTree.cpp:480-485)
  virtual void UpdateActiveParticleCounters(Hydrodynamics<ndim>* hydro) {
    check(gsph_update_active_particle_counters(ctx_, hydro->template GetParticleArray<ParticleType>(),
                                               hydro->Nhydro, sizeof(P), &off_));
  }

  // HydroTree::GetMaximumSmoothingLength (src/Tree/HydroTree.cpp:661-671)
  virtual double GetMaximumSmoothingLength() const {
    double h = 0.0;
    if (gsph_get_maximum_smoothing_length(ctx_, &h) != GSPH_OK)
      ExceptionHandler::getIstance().raise(gsph_last_error(ctx_));
    return h;
  }

  // GradhSphTree::UpdateAllSphProperties (src/GradhSph/GradhSphTree.cpp:82-271)
  virtual void UpdateAllSphProperties(Sph<ndim>* sph, Nbody<ndim>*) {
    check(gsph_update_all_sph_properties(ctx_));
    write_back(sph);
  }
  // GradhSphTree::UpdateAllSphHydroForces (src/GradhSph/GradhSphTree.cpp:279-435)
  virtual void UpdateAllSphHydroForces(Sph<ndim>* sph, Nbody<ndim>*, DomainBox<ndim>&) {
    check(gsph_update_all_sph_hydro_forces(ctx_));
    write_back(sph);
  }
  // GradhSphTree::UpdateAllSphForces (src/GradhSph/GradhSphTree.cpp:443-657); periodic
  // self-gravity (Ewald) is outside the library's path and reported as unsupported
  virtual void UpdateAllSphForces(Sph<ndim>* sph, Nbody<ndim>*, DomainBox<ndim>&, Ewald<ndim>*) {
    check(gsph_update_all_sph_forces(ctx_));
    write_back(sph);
  }

  gsph_ctx* context() const { return ctx_; }

 private:
  gsph_ctx* ctx_ = nullptr;
  gsph_field_offsets off_;

  void check(int rc) {
    if (rc != GSPH_OK) ExceptionHandler::getIstance().raise(gsph_last_error(ctx_));
  }
  void write_back(Sph<ndim>* sph) {
    check(gsph_get_particles_aos(ctx_, sph->template GetParticleArray<ParticleType>(), sph->Nhydro, sizeof(P),
                                 &off_));
  }
};

#endif  // GPU_GRADH_SPH_TREE_HPP_
