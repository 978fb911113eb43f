// Compile-only check (test infrastructure): the GANDALF-side drop-in
// include/gpu_gradh_sph_tree.hpp against the reference's own headers, instantiated for the
// library's path (3-D GradhSphParticle).  Built with -fsyntax-only by
// `make -f oracle/Makefile.ref integration-check`; nothing is linked or run.
#include "gpu_gradh_sph_tree.hpp"

template class GpuGradhSphTree<3, GradhSphParticle>;

// The subclass must stand in wherever the simulation keeps its neighbour search.
SphNeighbourSearch<3>* as_neighbour_search(GpuGradhSphTree<3, GradhSphParticle>* t) { return t; }
