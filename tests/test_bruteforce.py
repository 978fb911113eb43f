"""SPH neighbour sets against an O(N^2) brute-force search.

The reference's hydro membership (NeighbourManager.h:521) is |r_j - r_i|^2 < 4 h_i^2 or
< 4 h_j^2, with the periodic minimum image where the box is periodic; the particle
itself is a member.  The search below applies that predicate to every pair, with the
smoothing lengths the run produced, and must give exactly the lists the reference's tree
walk built (fixtures) and the lists the GPU built (both forms).
"""
import numpy as np
import pytest

from gandalf_gb300 import ics as ics_mod
from parity import csr_lists, load_golden, same_lists


def brute_force_lists(c, params, hrangesqd):
    x = np.stack([c["x"], c["y"], c["z"]], 1)
    periodic = bool(params.get("periodic", 0))
    if periodic:
        lo = np.asarray(params["boxmin"], dtype=np.float64)
        size = np.asarray(params["boxmax"], dtype=np.float64) - lo
    out = []
    for i in range(len(x)):
        dr = x - x[i]
        if periodic:
            dr = dr - size * np.round(dr / size)
        d2 = (dr[:, 0] * dr[:, 0] + dr[:, 1] * dr[:, 1]) + dr[:, 2] * dr[:, 2]
        out.append(np.where((d2 < hrangesqd[i]) | (d2 < hrangesqd))[0].astype(np.int32))
    return out


@pytest.mark.parametrize("name", ["cube2048", "plummer2048"])
def test_reference_lists_are_brute_force_complete(name):
    ics, params, ref, d = load_golden(name)
    assert same_lists(brute_force_lists(ics, params, ref["hrangesqd"]),
                      csr_lists(d["hydro_off"], d["hydro_ids"])) == []


def test_brute_force_sees_a_planted_mistake():
    ics, params, ref, d = load_golden("plummer2048")
    hr = ref["hrangesqd"].copy()
    hr[17] *= 1.5
    assert same_lists(brute_force_lists(ics, params, hr), csr_lists(d["hydro_off"], d["hydro_ids"])) != []


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("workload,n", [("plummer_sphere", 4099), ("periodic_cube", 4096)])
def test_gpu_lists_are_brute_force_complete(precision, workload, n):
    from gandalf_gb300.sph import GradhSphTree
    c = ics_mod.WORKLOADS[workload](n)
    params = c.pop("params")
    t = GradhSphTree(params, precision=precision)
    t.set_particles(c)
    t.set_recording(True, 4096)
    t.step()
    out = t.results()
    assert same_lists(t.sph_neighbours(), brute_force_lists(c, params, out["hrangesqd"])) == []
    t.close()
