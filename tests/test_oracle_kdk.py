"""The oracle's KDK main loop (block timesteps, active particles) against the reference.

The fixtures hold the reference's state after SetupSimulation and several MainLoop steps
(SphLeapfrogKDK, ComputeBlockTimesteps, CheckTimesteps), produced by the reference itself:
a rotating isothermal cloud with self-gravity (4 levels) and an adiabatic periodic cube
(3 levels, energy equation).  The discrete state (integer time, levels, step lengths,
neighbour levels) must agree exactly; positions, velocities and solved fields within a few
1e-10 (FP64 summation-order differences carried through the steps).
"""
import numpy as np
import pytest

from oracle import oracle
from parity import GOLDEN, INPUT_KEYS

KDK_KEYS = ("nlevels", "level_diff_max", "courant_mult", "accel_mult", "energy_mult")


def load(name):
    d = np.load(f"{GOLDEN}/{name}.npz")
    c = {k: d[k] for k in INPUT_KEYS}
    params = {k[6:]: d[k].tolist() for k in d.files if k.startswith("param_")}
    kdk = {k[4:]: d[k].tolist() for k in d.files if k.startswith("kdk_")}
    ref = {k: d["state"][:, i] for i, k in enumerate(oracle.KDK_FIELDS)}
    glob = {k: float(d["global"][i]) for i, k in enumerate(oracle.KDK_GLOBAL)}
    return c, params, kdk, ref, glob


def rel(a, b):
    s = np.abs(b) + 1e-6 * np.sqrt(np.mean(b * b)) + 1e-300
    return float(np.max(np.abs(a - b) / s))


@pytest.mark.parametrize("name", ["rotating_kdk2048", "cube_kdk2048"])
def test_oracle_kdk_matches_reference_main_loop(name):
    c, params, kdk, ref, glob = load(name)
    r = oracle.kdk(c, params, {k: kdk[k] for k in KDK_KEYS}, kdk["nsteps"], nthreads=2)
    assert r["status"] == 0
    g = r["global"]
    for k in ("n", "nresync", "Nsteps", "level_max", "level_step"):
        assert g[k] == glob[k], (k, g[k], glob[k])
    for k in ("t", "timestep", "dt_max"):
        assert abs(g[k] - glob[k]) <= 1e-10 * abs(glob[k]), (k, g[k], glob[k])
    out = r["state"]
    for k in ("level", "nstep", "nlast", "levelneib"):
        np.testing.assert_array_equal(out[k], ref[k], err_msg=k)
    for k in ("dt", "tlast"):
        assert rel(out[k], ref[k]) <= 1e-10, k
    for k in ("x", "y", "z"):
        assert np.max(np.abs(out[k] - ref[k])) <= 1e-10, k
    for k, tol in (("vx", 1e-9), ("vy", 1e-9), ("vz", 1e-9), ("h", 1e-10), ("rho", 1e-10), ("u", 1e-10),
                   ("ax", 1e-8), ("ay", 1e-8), ("az", 1e-8), ("dudt", 1e-8), ("gpot", 1e-10),
                   ("invomega", 1e-9), ("pressure", 1e-10), ("sound", 1e-10)):
        assert rel(out[k], ref[k]) <= tol, (k, rel(out[k], ref[k]))
    # block timesteps really were exercised: several levels, and fewer active updates
    # than a full-activity run would have
    assert len(np.unique(out["level"])) >= 2
    assert 0 < r["step_updates"] < kdk["nsteps"] * len(c["x"])


def test_oracle_kdk_detects_a_planted_mistake():
    """A one-ulp-scale change in a velocity must move the state away from the fixture."""
    c, params, kdk, ref, _ = load("rotating_kdk2048")
    bad = dict(c)
    bad["vx"] = c["vx"] + 1e-6 * np.std(c["vx"])
    r = oracle.kdk(bad, params, {k: kdk[k] for k in KDK_KEYS}, kdk["nsteps"], nthreads=2)
    assert np.max(np.abs(r["state"]["x"] - ref["x"])) > 1e-10
