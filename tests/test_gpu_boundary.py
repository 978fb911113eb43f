"""The drop-in boundary with block timesteps: GANDALF's particle records through the C ABI
in the order SphSimulation::MainLoop calls the neighbour search
(src/Hydrodynamics/SphSimulation.cpp:634-752), against the oracle given the same active
particles.

A previous step's solved state sits in the records; positions have drifted; about a
quarter of the particles are active, with random timestep levels.  The calls must solve
and write the active particles only, leave every other byte of the records as the caller
has it (host edits between calls included), and update levelneib of every particle as the
reference's force loops do.  Both transfer paths are covered: page-locked records (read and
written in place by kernels) and pageable ones (staged copies).
"""
import numpy as np
import pytest

from gandalf_gb300 import ics as ics_mod
from gandalf_gb300.sph import GradhSphTree
from oracle import oracle
from parity import FP64_TOL, assert_close, assert_vec_close, gradh_record_dtype

pytestmark = pytest.mark.gpu

OFFSET_KEYS = ("r", "v", "m", "h", "u", "rho", "invomega", "zeta", "hfactor", "hrangesqd", "pressure", "sound",
               "div_v", "dudt", "a", "atree", "gpot", "gpot_hydro", "flags", "level", "levelneib")
POTMIN = 1 << 3          # another reference flag bit: must be ignored and kept


def offsets(dt):
    return {k: dt.fields[k][1] for k in OFFSET_KEYS}


def records(n, pinned):
    dt = gradh_record_dtype()
    if pinned:
        import torch
        buf = torch.zeros(n * dt.itemsize, dtype=torch.uint8).pin_memory()
        return buf, buf.numpy().view(dt)
    return None, np.zeros(n, dtype=dt)


def scenario(name, seed):
    """Particles after a drift from a solved state, with an active mask and levels."""
    c = ics_mod.plummer_sphere(6000, seed=seed) if name == "plummer" else ics_mod.periodic_cube(4096, seed=seed)
    params = c.pop("params")
    solved = oracle.run(c, params, nthreads=4)["particles"]
    rng = np.random.default_rng(seed)
    n = len(c["x"])
    x = np.stack([c["x"], c["y"], c["z"]], 1)
    v = np.stack([c["vx"], c["vy"], c["vz"]], 1)
    dt = 0.05 * np.median(solved["h"] / (np.linalg.norm(v, axis=1) + solved["sound"]))
    x = x + dt * v
    if params.get("periodic"):
        lo, hi = np.array(params["boxmin"]), np.array(params["boxmax"])
        x = lo + np.mod(x - lo, hi - lo)
    act = rng.random(n) < 0.25
    level = rng.integers(0, 4, n).astype(np.int32)
    lvn = rng.integers(0, 4, n).astype(np.int32)
    return c, params, solved, x, v, act, level, lvn, rng


def fill(rec, c, solved, x, v, act, level, lvn, rng):
    rec["r"] = x
    rec["v"] = v
    rec["m"], rec["u"], rec["h"] = c["m"], solved["u"], solved["h"]
    for k in ("rho", "invomega", "zeta", "hfactor", "hrangesqd", "pressure", "sound", "div_v", "dudt", "gpot",
              "gpot_hydro"):
        rec[k] = solved[k]
    rec["a"] = np.stack([solved["ax"], solved["ay"], solved["az"]], 1)
    rec["atree"] = np.stack([solved["agx"], solved["agy"], solved["agz"]], 1)
    rec["flags"] = np.where(act, 2, 0).astype(np.uint32) | np.where(rng.random(len(act)) < 0.3, POTMIN, 0).astype(np.uint32)
    rec["level"] = level
    rec["levelneib"] = lvn
    rec["iorig"] = np.arange(len(act))
    rec["ionfrac"] = rng.random(len(act))
    rec["r0"] = rng.random((len(act), 3))
    rec["alpha"] = 1.0


def zero_accelerations(rec, act):
    """Sph::ZeroAccelerations for the active particles (src/Hydrodynamics/Sph.cpp:126-140)."""
    rec["levelneib"][act] = 0
    for k in ("div_v", "dudt", "gpot", "gpot_hydro"):
        rec[k][act] = 0.0
    rec["a"][act] = 0.0
    rec["atree"][act] = 0.0


def check_active(rec, ref, act, gravity):
    got = {k: rec[k][act] for k in ("h", "rho", "pressure", "sound", "hfactor", "invomega", "zeta", "div_v", "dudt")}
    for k, v in got.items():
        assert_close(k, v, ref[k][act], FP64_TOL[k])
    assert_vec_close("a", tuple(rec["a"][act].T), tuple(ref[k][act] for k in ("ax", "ay", "az")), FP64_TOL["a"])
    if gravity:
        assert_vec_close("atree", tuple(rec["atree"][act].T), tuple(ref[k][act] for k in ("agx", "agy", "agz")),
                         FP64_TOL["ag"])
        assert_close("gpot", rec["gpot"][act], ref["gpot"][act], FP64_TOL["gpot"])


def same_bytes_except(a, b, mask, skip=("levelneib",)):
    """Records a and b equal byte for byte on the masked rows, apart from `skip` fields."""
    for name in a.dtype.names:
        if name in skip:
            continue
        if not np.array_equal(a[name][mask], b[name][mask]):
            return name
    return None


@pytest.mark.parametrize("name", ["plummer", "cube"])
@pytest.mark.parametrize("pinned", [True, False])
def test_main_loop_order_with_active_particles(name, pinned):
    c, params, solved, x, v, act, level, lvn, rng = scenario(name, 11 if name == "plummer" else 12)
    gravity = bool(params.get("self_gravity"))
    n = len(act)
    buf, rec = records(n, pinned)
    fill(rec, c, solved, x, v, act, level, lvn, rng)
    off = offsets(rec.dtype)
    t = GradhSphTree(params)
    t.set_particles_aos(rec, off)
    t.BuildTree()
    hmax_tree = t.GetMaximumSmoothingLength()
    assert hmax_tree == pytest.approx(float(np.max(rec["h"])), rel=0, abs=0)
    t.UpdateAllSphProperties()
    before = rec.copy()
    t.get_particles_aos(rec, off)
    # nothing of an inactive record changed
    assert same_bytes_except(rec, before, ~act, skip=()) is None
    # the caller's work between the passes, as MainLoop does, plus unrelated edits
    zero_accelerations(rec, act)
    rec["dt"] = 42.0
    rec["ionfrac"] += 1.0
    snap = rec.copy()
    if gravity:
        t.UpdateAllSphForces()
    else:
        t.UpdateAllSphHydroForces()
    t.get_particles_aos(rec, off)
    t.close()
    # oracle: the same pass given the same active particles and state
    ics = {"x": x[:, 0], "y": x[:, 1], "z": x[:, 2], "vx": v[:, 0], "vy": v[:, 1], "vz": v[:, 2],
           "m": c["m"], "u": solved["u"], "h": solved["h"]}
    ap = oracle.ActivePasses(params, nthreads=4)
    ref = ap.run(ics, act, level, snap["levelneib"], {k: solved[k] for k in oracle.STATE_FIELDS})
    ap.close()
    check_active(rec, ref, act, gravity)
    np.testing.assert_array_equal(rec["levelneib"], ref["levelneib"])
    assert np.any(rec["levelneib"] != snap["levelneib"])          # the pass did raise some
    # inactive records: untouched apart from levelneib; host edits kept everywhere
    assert same_bytes_except(rec, snap, ~act) is None
    assert np.all(rec["dt"] == 42.0)
    np.testing.assert_array_equal(rec["ionfrac"], snap["ionfrac"])
    np.testing.assert_array_equal(rec["flags"], snap["flags"])
    np.testing.assert_array_equal(rec["r0"], snap["r0"])


def test_repeated_pass_after_check_timesteps():
    """MainLoop's repeat (SphSimulation.cpp:641-752): after CheckTimesteps activates more
    particles, UpdateActiveParticleCounters and a second h solve + force pass on the same
    tree.  Hydro only (the periodic cube), so the results do not depend on the tree."""
    c, params, solved, x, v, act, level, lvn, rng = scenario("cube", 13)
    n = len(act)
    buf, rec = records(n, True)
    fill(rec, c, solved, x, v, act, level, lvn, rng)
    off = offsets(rec.dtype)
    ics = {"x": x[:, 0], "y": x[:, 1], "z": x[:, 2], "vx": v[:, 0], "vy": v[:, 1], "vz": v[:, 2],
           "m": c["m"], "u": solved["u"], "h": solved["h"]}
    ap = oracle.ActivePasses(params, nthreads=4)
    t = GradhSphTree(params)
    t.set_particles_aos(rec, off)
    t.BuildTree()
    t.UpdateAllSphProperties()
    t.get_particles_aos(rec, off)
    zero_accelerations(rec, act)
    lvn0 = rec["levelneib"].copy()
    t.UpdateAllSphHydroForces()
    t.get_particles_aos(rec, off)
    ref1 = ap.run(ics, act, level, lvn0, {k: solved[k] for k in oracle.STATE_FIELDS})
    check_active(rec, ref1, act, False)
    # CheckTimesteps on the host: unset active, activate a new set
    act2 = (~act) & (rng.random(n) < 0.2)
    rec["flags"] = (rec["flags"] & ~np.uint32(2)) | np.where(act2, 2, 0).astype(np.uint32)
    rec["level"][act2] += 1
    t.UpdateActiveParticleCounters(rec, off)
    state2 = {k: rec[k].copy() for k in oracle.STATE_FIELDS}
    ics2 = dict(ics)
    ics2["h"] = rec["h"].copy()
    t.UpdateAllSphProperties()
    t.get_particles_aos(rec, off)
    zero_accelerations(rec, act2)
    lvn1 = rec["levelneib"].copy()
    snap = rec.copy()
    t.UpdateAllSphHydroForces()
    t.get_particles_aos(rec, off)
    t.close()
    ref2 = ap.run(ics2, act2, rec["level"], lvn1, state2, rebuild=False)
    ap.close()
    check_active(rec, ref2, act2, False)
    np.testing.assert_array_equal(rec["levelneib"], ref2["levelneib"])
    assert same_bytes_except(rec, snap, ~act2) is None
