"""Mixed-precision form (fp32 pair arithmetic) against the fp64 oracle and fixtures.

* h solve: h, rho, Omega^-1, P against the full fp64 oracle, MIXED_TOL (rms relative
  error <= 1e-4 as the target states; typical 1e-7).
* Interaction lists: every membership decision is made with the reference's fp64
  arithmetic whenever the float value is inside the margin, so the lists are those the
  reference's criteria give for the mixed form's own smoothing lengths — checked
  bit-exactly against the oracle run with those h values supplied.  (Its h differ from
  the fp64 form's by ~1e-7, so pairs or cells within ~1e-7 of a threshold can differ
  from the fp64 lists; the full-size test reports how many.)
* Forces: against the oracle given the same h (the force pass alone) and against the
  full fp64 oracle, MIXED_TOL.
"""
import numpy as np
import pytest

from gandalf_gb300 import ics as ics_mod
from gandalf_gb300.sph import GradhSphTree
from oracle import oracle
from parity import check_mixed, load_golden, same_lists

pytestmark = pytest.mark.gpu

SOLVED = ("h", "rho", "invomega", "zeta", "pressure", "sound")


def run_mixed(c, params, record=True):
    t = GradhSphTree(params, precision="mixed")
    t.set_particles(c)
    if record:
        t.set_recording(True, 4096)
    t.step()
    return t, t.results()


def check_against_oracle(c, params, full_ref=None):
    t, out = run_mixed(c, params)
    full = full_ref if full_ref is not None else oracle.run(c, params)["particles"]
    dens = check_mixed({k: out[k] for k in ("h", "rho", "pressure", "invomega")},
                       {k: full[k] for k in ("h", "rho", "pressure", "invomega")})
    r = oracle.run(c, params, summary=True, given={k: out[k] for k in SOLVED})
    assert same_lists(t.sph_neighbours(), r["hydro_neib"]) == []
    gravity = bool(params.get("self_gravity"))
    if gravity:
        cnt, hsh = t.direct_summary()
        assert np.array_equal(cnt, r["direct_count"])
        assert np.array_equal(hsh, r["direct_hash"])
        leaf, ccnt, chsh = t.cell_summary()
        assert np.array_equal(leaf, r["leaf_cell"])
        assert np.array_equal(ccnt, r["cell_count"])
        assert np.array_equal(chsh, r["cell_hash"])
    force_keys = ("ax", "ay", "az", "agx", "agy", "agz", "gpot", "dudt", "div_v")
    forces = check_mixed({k: out[k] for k in force_keys}, {k: r["particles"][k] for k in force_keys})
    total = check_mixed(out, full)
    st = t.stats()
    t.close()
    return dens, forces, total, st


@pytest.mark.parametrize("name", ["cube2048", "plummer2048"])
def test_mixed_fixture(name):
    ics, params, ref, d = load_golden(name)
    print(name, check_against_oracle(ics, params, full_ref=ref))


@pytest.mark.parametrize("n,seed", [(4099, 4190), (65536, 65627), (65536, 65613)])
def test_mixed_plummer_vs_oracle(n, seed):
    c = ics_mod.plummer_sphere(n, seed=seed)
    print(n, check_against_oracle(c, c["params"]))


def test_mixed_periodic_cube_full_size():
    c = ics_mod.periodic_cube(32768, seed=1234)
    print(check_against_oracle(c, c["params"]))


def test_mixed_plummer_full_size():
    """The bench workload: mixed against the oracle (h solve, lists, forces) and the
    number of list entries that differ from the fp64 GPU form's lists."""
    c = ics_mod.plummer_sphere(262144, seed=4321)
    dens, forces, total, st = check_against_oracle(c, c["params"])
    b = GradhSphTree(c["params"], precision="fp64")
    b.set_particles(c)
    b.set_recording(True, 4096)
    b.step()
    a = GradhSphTree(c["params"], precision="mixed")
    a.set_particles(c)
    a.set_recording(True, 4096)
    a.step()
    d_sph = len(same_lists(a.sph_neighbours(), b.sph_neighbours()))
    d_cells = int(np.sum(a.cell_summary()[1] != b.cell_summary()[1]))
    print({"h_solve": dens, "forces": forces, "total": total, "particles_with_other_sph_list": d_sph,
           "leaves_with_other_cell_count": d_cells, "stats": st})
    assert d_sph <= 1e-4 * len(c["x"]) and d_cells <= 1e-3 * st["nleaf"]


def test_mixed_compensated_sums():
    """The compensated form (Kahan float sums, lane partials combined in FP64) against the
    full fp64 oracle at tight h_converge, where the iteration path is the same in every
    form and the remaining difference is the pair arithmetic: within MIXED_TOL, no worse
    than the plain float sums in rho, and the switch changes the results."""
    c = ics_mod.plummer_sphere(65536, seed=65601)
    params = dict(c["params"], h_converge=1e-10)
    full = oracle.run(c, params)["particles"]
    res = {}
    for comp in (0, 1):
        t = GradhSphTree(params, precision="mixed", compensated=comp)
        t.set_particles(c)
        t.step()
        res[comp] = t.results()
        t.close()
    plain = check_mixed(res[0], full)
    comp = check_mixed(res[1], full)
    print({"plain": plain, "compensated": comp})
    assert not np.array_equal(res[0]["rho"], res[1]["rho"])
    assert comp["rho"][0] <= 1.5 * plain["rho"][0]
    assert comp["ag_nrms"] <= 1.5 * plain["ag_nrms"]
