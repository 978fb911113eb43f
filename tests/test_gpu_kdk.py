"""KDK leapfrog with block timesteps on the GPU against the reference's own main loop.

The fixtures hold the reference's state after SetupSimulation and several MainLoop steps
(SphLeapfrogKDK, ComputeBlockTimesteps, CheckTimesteps): a rotating isothermal cloud with
self-gravity (4 levels) and an adiabatic periodic cube (3 levels, energy equation).  The
discrete state (integer time, levels, step lengths) must agree exactly; positions,
velocities and solved fields to a few 1e-10 (the FP64 differences of summation order,
carried through the steps).
"""
import numpy as np
import pytest

from gandalf_gb300 import ics as ics_mod
from gandalf_gb300.sph import GradhSphTree
from parity import GOLDEN, INPUT_KEYS

pytestmark = pytest.mark.gpu

KDK_FIELDS = ["x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az", "h", "rho", "u", "level", "nstep", "nlast",
              "levelneib", "dt", "tlast", "dudt", "div_v", "gpot", "invomega", "pressure", "sound"]
KDK_GLOBAL = ["n", "t", "timestep", "level_max", "level_step", "nresync", "Nsteps", "dt_max"]


def load(name):
    d = np.load(f"{GOLDEN}/{name}.npz")
    c = {k: d[k] for k in INPUT_KEYS}
    params = {k[6:]: d[k].tolist() for k in d.files if k.startswith("param_")}
    kdk = {k[4:]: d[k].tolist() for k in d.files if k.startswith("kdk_")}
    ref = {k: d["state"][:, i] for i, k in enumerate(KDK_FIELDS)}
    glob = {k: float(d["global"][i]) for i, k in enumerate(KDK_GLOBAL)}
    return c, params, kdk, ref, glob


def run(c, params, kdk, precision="fp64", graph=True, nsteps=None):
    t = GradhSphTree(params, precision=precision)
    t.set_particles(c)
    cfg = {k: kdk[k] for k in ("nlevels", "level_diff_max", "courant_mult", "accel_mult", "energy_mult")}
    t.kdk_setup(**cfg)
    t.kdk_steps(nsteps or kdk["nsteps"], graph=graph)
    out = {k: t.kdk_state(k) for k in ("x", "y", "z", "vx", "vy", "vz", "u", "dt", "tlast", "level", "nstep",
                                       "nlast", "levelneib")}
    res = t.results()
    for k in ("ax", "ay", "az", "h", "rho", "dudt", "div_v", "gpot", "invomega", "pressure", "sound"):
        out[k] = res[k]
    st = t.kdk_status()
    t.close()
    return out, st


def rel(a, b, scale=None):
    s = np.abs(b) + (scale if scale is not None else 1e-6 * np.sqrt(np.mean(b * b)) + 1e-300)
    return float(np.max(np.abs(a - b) / s))


@pytest.mark.parametrize("name", ["rotating_kdk2048", "cube_kdk2048"])
def test_kdk_matches_reference(name):
    c, params, kdk, ref, glob = load(name)
    out, st = run(c, params, kdk)
    assert st["status"] == 0
    assert st["n"] == glob["n"] and st["nresync"] == glob["nresync"] and st["nsteps"] == glob["Nsteps"]
    assert st["level_max"] == glob["level_max"] and st["level_step"] == glob["level_step"]
    for k in ("t", "timestep", "dt_max"):
        assert abs(st[k] - glob[k]) <= 1e-10 * abs(glob[k]), (k, st[k], glob[k])
    for k in ("level", "nstep", "nlast", "levelneib"):
        np.testing.assert_array_equal(out[k], ref[k], err_msg=k)
    for k in ("dt", "tlast"):
        assert rel(out[k], ref[k]) <= 1e-10, k
    box = 1.0
    for k in ("x", "y", "z"):
        assert np.max(np.abs(out[k] - ref[k])) <= 1e-10 * box, k
    for k, tol in (("vx", 1e-9), ("vy", 1e-9), ("vz", 1e-9), ("h", 1e-10), ("rho", 1e-10), ("u", 1e-10),
                   ("ax", 1e-8), ("ay", 1e-8), ("az", 1e-8), ("dudt", 1e-8), ("gpot", 1e-10)):
        assert rel(out[k], ref[k]) <= tol, (k, rel(out[k], ref[k]))


def test_kdk_graph_equals_stream_launches():
    """The graph (CheckTimesteps repeat passes as conditional nodes, set on the device) and
    stream launches (the host reads whether a repeat pass has work) give identical states."""
    c, params, kdk, _, _ = load("rotating_kdk2048")
    a, sa = run(c, params, kdk, graph=True)
    b, sb = run(c, params, kdk, graph=False)
    for k in a:
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)
    assert sa == sb


def test_kdk_timing_of_first_passes():
    c = ics_mod.rotating_cloud(16384, seed=44)
    params = c.pop("params")
    kdk = c.pop("kdk")
    t = GradhSphTree(params, precision="mixed")
    t.set_particles(c)
    t.kdk_setup(**kdk)
    t.kdk_steps(4, graph=True)
    tm = t.kdk_timing()
    st = t.stats()
    t.close()
    assert tm["steps"] == 4 and tm["ms_forces"] > 0 and tm["ms_density"] > 0 and tm["ms_build"] > 0
    assert 0 < tm["hydro_pairs"] <= st["hydro_pairs"] and 0 < tm["cell_pairs"] <= st["cell_pairs"]
    assert 0 <= tm["repeat_passes"] <= 8


def test_kdk_mixed_tracks_fp64():
    c = ics_mod.rotating_cloud(32768, seed=43)
    params = c.pop("params")
    kdk = c.pop("kdk")
    a, sa = run(c, params, kdk, precision="fp64", nsteps=6)
    b, sb = run(c, params, kdk, precision="mixed", nsteps=6)
    assert sa["status"] == 0 and sb["status"] == 0
    same = np.mean(a["level"] == b["level"])
    assert same > 0.99, same
    for k in ("x", "y", "z"):
        assert np.sqrt(np.mean((a[k] - b[k]) ** 2)) <= 1e-6, k
    e = np.abs(a["rho"] - b["rho"]) / a["rho"]
    assert np.sqrt(np.mean(e * e)) <= 1e-4


def test_kdk_matches_oracle_main_loop_on_the_cloud():
    """The headline configuration's shape at 32,768 particles: setup plus 6 KDK steps of
    the rotating cloud (4 levels), FP64 GPU form against the oracle's main loop.  Levels,
    step lengths and neighbour levels exactly; positions and solved fields to FP64
    summation-order differences."""
    from oracle import oracle
    c = ics_mod.rotating_cloud(32768, seed=47)
    params = c.pop("params")
    kdk = c.pop("kdk")
    out, st = run(c, params, kdk, precision="fp64", nsteps=6)
    r = oracle.kdk(c, params, kdk, 6)
    ref, glob = r["state"], r["global"]
    assert st["status"] == 0 and r["status"] == 0
    assert st["n"] == glob["n"] and st["level_max"] == glob["level_max"] and st["nsteps"] == glob["Nsteps"]
    assert abs(st["t"] - glob["t"]) <= 1e-12 * abs(glob["t"])
    for k in ("level", "nstep", "nlast", "levelneib"):
        np.testing.assert_array_equal(out[k], ref[k], err_msg=k)
    for k in ("x", "y", "z"):
        assert np.max(np.abs(out[k] - ref[k])) <= 1e-10, k
    for k, tol in (("h", 1e-10), ("rho", 1e-10), ("ax", 1e-8), ("gpot", 1e-10)):
        assert rel(out[k], ref[k]) <= tol, (k, rel(out[k], ref[k]))
    # the active particle updates agree with the oracle's count
    assert st["active_updates"] == r["setup_updates"] + r["step_updates"]
