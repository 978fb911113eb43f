// Test infrastructure: prints the byte layout of the reference's GradhSphParticle<3>
// (src/Headers/Particle.h:133-368) as "field offset size" lines and "sizeof N", so the
// record layouts the tests and the bench build in numpy can be checked against the
// reference's own compiler layout.  Built by `make -f oracle/Makefile.ref record-layout`.
#include <cstddef>
#include <cstdio>

#include "Particle.h"

#define FIELD(name) std::printf("%s %zu %zu\n", #name, offsetof(P, name), sizeof(((P*) nullptr)->name))

int main() {
  typedef GradhSphParticle<3> P;
  FIELD(flags); FIELD(ptype); FIELD(iorig); FIELD(sinkid); FIELD(levelneib); FIELD(nstep); FIELD(nlast);
  FIELD(level); FIELD(r); FIELD(v); FIELD(a); FIELD(atree); FIELD(r0); FIELD(v0); FIELD(a0); FIELD(m); FIELD(h);
  FIELD(h_dust); FIELD(hrangesqd); FIELD(hfactor); FIELD(sound); FIELD(rho); FIELD(pressure); FIELD(u); FIELD(u0);
  FIELD(dudt0); FIELD(dudt); FIELD(gpot); FIELD(gpot_hydro); FIELD(dt); FIELD(dt_next); FIELD(tlast);
  FIELD(ionfrac); FIELD(Xion); FIELD(ueq); FIELD(dt_therm); FIELD(vsig_max); FIELD(rad_pres); FIELD(ionstate);
  FIELD(div_v); FIELD(alpha); FIELD(dalphadt); FIELD(invomega); FIELD(zeta);
  std::printf("sizeof %zu\n", sizeof(P));
  return 0;
}
