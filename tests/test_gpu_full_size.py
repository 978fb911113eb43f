"""Full-size workloads on the GPU: parity with the oracle plus size-independent checks.

Grad-h SPH pair forces are antisymmetric, so sum_i m_i a_hydro,i vanishes and
sum_i m_i (v_i . a_hydro,i + du_i/dt) vanishes (energy conservation of the hydro
terms) to rounding: |sum| / sum |terms| <= 1e-10 is asserted.
"""
import numpy as np
import pytest

from gandalf_gb300 import ics as ics_mod
from gandalf_gb300.sph import GradhSphTree
from oracle import oracle
from parity import check_fp64

pytestmark = pytest.mark.gpu


def conservation(c, out):
    m = c["m"]
    ah = np.stack([out["ax"] - out["agx"], out["ay"] - out["agy"], out["az"] - out["agz"]], 1)
    mom = (m[:, None] * ah).sum(0)
    mom_scale = (m[:, None] * np.abs(ah)).sum(0)
    v = np.stack([c["vx"], c["vy"], c["vz"]], 1)
    power = m * ((v * ah).sum(1) + out["dudt"])
    return np.abs(mom) / mom_scale, abs(power.sum()) / np.abs(m * out["dudt"]).sum()


def test_plummer_full_size_fp64():
    """The Plummer workload at N = 262144: oracle parity and hydro conservation."""
    c = ics_mod.plummer_sphere(262144, seed=4321)
    t = GradhSphTree(c["params"])
    t.set_particles(c)
    t.step()
    out = t.results()
    r = oracle.run(c, c["params"])
    check_fp64(out, r["particles"], gravity=True)
    mom, power = conservation(c, out)
    assert np.all(mom < 1e-10), mom
    assert power < 1e-10, power
    st = t.stats()
    assert st["status"] == 0
    assert st["direct_pairs"] == r["counts"]["direct_pairs"]
    assert st["cell_pairs"] == r["counts"]["cell_pairs"]


def test_cube_full_size_conservation():
    c = ics_mod.periodic_cube(32768, seed=1234)
    t = GradhSphTree(c["params"])
    t.set_particles(c)
    t.step()
    out = t.results()
    mom, power = conservation(c, out)
    assert np.all(mom < 1e-10), mom
    assert power < 1e-10, power
