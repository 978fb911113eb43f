"""Star-gas coupling on the GPU against the reference fixture and the oracle.

Gas <- stars: the stars' softened gravity in a, atree and gpot, gpot_hydro without it,
and the SPH-star zeta term of the h solve.  Star <- gas: a, adot and gpot of every star
from the gas tree.  FP64 form: FP64_TOL and STAR_TOL of tests/parity.py.  Mixed form:
its gas fields within MIXED_TOL; the star pass is FP64 arithmetic on the mixed form's
smoothing lengths (float h iteration, h within MIXED_TOL), within 1e-5.
"""
import numpy as np
import pytest

from gandalf_gb300 import ics as ics_mod
from gandalf_gb300.sph import GradhSphTree
from oracle import oracle
from parity import (assert_close, assert_vec_close, check_fp64, check_mixed, check_stars, load_golden,
                    star_results)

pytestmark = pytest.mark.gpu


def run(ics, params, precision="fp64"):
    t = GradhSphTree(params, precision=precision)
    t.set_particles(ics)
    t.step()
    out = t.results()
    stars = t.star_forces() if params.get("self_gravity") else None
    t.close()
    return out, stars


def test_stars_match_reference_fixture():
    ics, params, ref, d = load_golden("plummer_stars2048")
    out, stars = run(ics, params)
    check_fp64(out, ref, True)
    assert_close("gpot_hydro", out["gpot_hydro"], ref["gpot_hydro"], 1e-11)
    check_stars(stars, star_results(d))


@pytest.mark.parametrize("n,nstar", [(65536, 64), (20000, 7)])
def test_stars_match_oracle(n, nstar):
    c = ics_mod.with_stars(ics_mod.plummer_sphere(n, seed=77), nstar, h=0.02, sigma_v=0.2, seed=78)
    params = c.pop("params")
    r = oracle.run(c, params)
    out, stars = run(c, params)
    check_fp64(out, r["particles"], True)
    assert_close("gpot_hydro", out["gpot_hydro"], r["particles"]["gpot_hydro"], 1e-11)
    check_stars(stars, r["stars"])
    mo, ms = run(c, params, precision="mixed")
    check_mixed(mo, r["particles"])
    for k in ("ax", "ay", "az", "gpot"):
        assert_close("mixed star " + k, ms[k], r["stars"][k], 1e-5)


def test_hydro_only_gas_feels_stars():
    c = ics_mod.periodic_cube(4096, seed=5)
    params = c.pop("params")
    rng = np.random.default_rng(6)
    c["stars"] = {"x": rng.random(3), "y": rng.random(3), "z": rng.random(3), "vx": np.zeros(3),
                  "vy": np.zeros(3), "vz": np.zeros(3), "m": np.full(3, 1e-3), "h": np.full(3, 0.05)}
    r = oracle.run(c, params)
    out, _ = run(c, params)
    check_fp64(out, r["particles"], True)
    assert np.abs(out["gpot"]).max() > 0


def test_removing_stars_restores_the_gas_only_result():
    c = ics_mod.with_stars(ics_mod.plummer_sphere(4099, seed=3), 8, h=0.05, seed=4)
    params = c.pop("params")
    gas = {k: v for k, v in c.items() if k != "stars"}
    t = GradhSphTree(params)
    t.set_particles(c)
    t.step()
    with_stars = t.results()
    t.set_stars(None)
    t.step()
    without = t.results()
    t.close()
    ref = oracle.run(gas, params)["particles"]
    check_fp64(without, ref, True)
    assert np.abs(with_stars["gpot"] - without["gpot"]).max() > 1e-6


def test_evrard_sphere_with_stars_against_oracle():
    """The Evrard configuration's shape at a seeded smaller N: a rho ~ 1/r gas sphere of
    65,536 particles with 64 stars (m = 1e-3, uniform in r < 0.5), FP64 form against the
    oracle at the FP64 tolerances, mixed form within MIXED_TOL and its star <- gas forces
    within 1e-5."""
    c = ics_mod.evrard_sphere(65536, seed=53, nstar=64)
    params = c.pop("params")
    r = oracle.run(c, params)
    out, stars = run(c, params)
    check_fp64(out, r["particles"], True)
    assert_close("gpot_hydro", out["gpot_hydro"], r["particles"]["gpot_hydro"], 1e-11)
    check_stars(stars, r["stars"])
    mo, ms = run(c, params, precision="mixed")
    print(check_mixed(mo, r["particles"]))
    for k in ("ax", "ay", "az", "gpot"):
        assert_close("mixed star " + k, ms[k], r["stars"][k], 1e-5)
