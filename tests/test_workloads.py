"""The seeded synthetic workloads have the shapes the benchmark configurations name.

CPU only: the generators of gandalf_gb300/ics.py are checked against the analytic
properties of each setup (mass profiles, energies, density contrasts, ranges), at sizes
where the sampling noise is well below the tolerances used.
"""
import math

import numpy as np

from gandalf_gb300 import ics as ics_mod


def radii(c):
    return np.sqrt(c["x"] ** 2 + c["y"] ** 2 + c["z"] ** 2)


def test_periodic_cube():
    c = ics_mod.periodic_cube(20000, seed=3)
    for k in ("x", "y", "z"):
        assert c[k].min() >= 0.0 and c[k].max() < 1.0
    assert np.isclose(c["m"].sum(), 1.0)
    assert np.all(np.abs(c["u"] - 1.0) <= 0.01)
    assert abs(np.std(c["vx"]) - 0.1) < 0.005
    assert c["params"]["periodic"] == 1 and c["params"]["self_gravity"] == 0


def test_plummer_mass_profile_and_bound_velocities():
    n = 200000
    c = ics_mod.plummer_sphere(n, seed=11)
    r = radii(c)
    assert r.max() <= 10.0 + 1e-9
    mass_frac = lambda x: x ** 3 / (1.0 + x * x) ** 1.5
    for x in (0.5, 1.0, 3.0):
        expect = mass_frac(x) / mass_frac(10.0)
        assert abs(np.mean(r < x) - expect) < 0.005, x
    v = np.sqrt(c["vx"] ** 2 + c["vy"] ** 2 + c["vz"] ** 2)
    vesc = math.sqrt(2.0) * (1.0 + r * r) ** -0.25
    assert np.all(v < vesc)
    # the Plummer distribution function is in virial equilibrium: K = |W| / 2 = 3 pi / 64
    # (the truncation at 10 scale radii changes K by less than the tolerance)
    kin = 0.5 * np.mean(v * v)
    assert abs(kin - 3.0 * math.pi / 64.0) < 0.01
    assert np.all(c["u"] == 0.05) and np.isclose(c["m"].sum(), 1.0)


def test_evrard_sphere_and_stars():
    n = 200000
    c = ics_mod.evrard_sphere(n, seed=5, nstar=64)
    r = radii(c)
    assert r.max() <= 1.0
    # rho ~ 1/r: M(<r) = r^2
    for x in (0.25, 0.5, 0.8):
        assert abs(np.mean(r < x) - x * x) < 0.005, x
    assert np.all(c["vx"] == 0.0) and np.all(c["u"] == 0.05)
    s = c["stars"]
    rs = np.sqrt(s["x"] ** 2 + s["y"] ** 2 + s["z"] ** 2)
    assert len(rs) == 64 and rs.max() < 0.5
    assert np.all(s["m"] == 1.0e-3) and np.all(s["h"] == 0.01)


def test_rotating_cloud_energies_and_perturbation():
    n = 400000
    c = ics_mod.rotating_cloud(n, seed=7)
    r = radii(c)
    assert r.max() <= 1.0
    assert abs(np.mean(r < 0.5) - 0.125) < 0.003            # uniform sphere
    m = c["m"]
    erot = 0.5 * np.sum(m * (c["vx"] ** 2 + c["vy"] ** 2))
    egrav = 3.0 / 5.0                                         # |E_grav| of the uniform sphere
    assert abs(erot / egrav - 0.16) < 0.003
    # isothermal: E_therm = (3/2) M c_s^2 = 0.26 |E_grav|
    p = c["params"]
    cs2 = p["temp0"] / p["mu_bar"]
    assert abs(1.5 * cs2 / egrav - 0.26) < 1e-12
    assert np.allclose(c["u"] * (p["gamma_eos"] - 1.0), cs2)
    # m = 2 perturbation rho ~ 1 + 0.1 cos(2 phi): <cos 2 phi> = 0.05
    phi = np.arctan2(c["y"], c["x"])
    assert abs(np.mean(np.cos(2.0 * phi)) - 0.05) < 0.004
    assert c["kdk"]["nlevels"] == 4


def test_kh_box_contrast_shear_pressure():
    n = 60000
    c = ics_mod.kh_box(n, seed=9)
    band = np.abs(c["y"] - 0.5) < 0.25
    assert abs(band.mean() - 2.0 / 3.0) < 0.01                 # 2:1 number density
    assert np.all(c["vx"][band] == -0.5) and np.all(c["vx"][~band] == 0.5)
    assert np.allclose(c["vy"], 0.01 * np.sin(4.0 * math.pi * c["x"]))
    rho = np.where(band, 2.0, 1.0)
    gamma = c["params"]["gamma_eos"]
    assert np.allclose((gamma - 1.0) * rho * c["u"], 2.5)        # uniform pressure
    assert c["z"].max() < 0.25 and c["params"]["boxmax"] == (1.0, 1.0, 0.25)


def test_kh_ensemble_sizes():
    boxes = ics_mod.kh_ensemble()
    sizes = np.array([len(b["x"]) for b in boxes])
    assert len(boxes) == 64
    assert sizes.min() >= 4096 and sizes.max() <= 131072
    assert 1.5e6 < sizes.sum() < 2.7e6


def test_leaf_size_tuner_reuses_its_cache(tmp_path):
    """A cached result for the same (N, precision, gravity, periodic) is returned without
    timing anything (no GPU needed)."""
    import json
    from gandalf_gb300.autotune import tune_leaf_size
    c = ics_mod.periodic_cube(1000, seed=1)
    params = c.pop("params")
    key = f"1000:mixed:{params['self_gravity']}:{params['periodic']}"
    cached = {"nleafmax": 12, "ms_per_step": {"8": 2.0, "12": 1.5}}
    path = tmp_path / "tune.json"
    path.write_text(json.dumps({key: cached}))
    assert tune_leaf_size(c, params, precision="mixed", cache=str(path)) == cached
