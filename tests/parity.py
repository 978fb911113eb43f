"""Comparison helpers shared by the parity tests (tolerances are stated per call)."""
from __future__ import annotations

import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
PARTICLE_FIELDS = ["h", "rho", "invomega", "zeta", "hfactor", "pressure", "sound", "u",
                   "div_v", "dudt", "ax", "ay", "az", "agx", "agy", "agz", "gpot",
                   "gpot_hydro", "hrangesqd", "levelneib"]
INPUT_KEYS = ("x", "y", "z", "vx", "vy", "vz", "m", "u", "h")


def load_golden(name):
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    ics = {k: d[k] for k in INPUT_KEYS}
    params = {k[6:]: d[k].tolist() for k in d.files if k.startswith("param_")}
    parts = {k: d["particles"][:, i] for i, k in enumerate(PARTICLE_FIELDS)}
    return ics, params, parts, d


def scaled_err(a, b):
    """|a - b| / (|b| + 1e-6 rms(b)): relative, with a floor for values near zero."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    floor = 1e-6 * np.sqrt(np.mean(b * b)) + 1e-300
    return np.abs(a - b) / (np.abs(b) + floor)


def vec_err(ax, ay, az, bx, by, bz):
    """Per-particle |a - b| / (|b| + 1e-6 rms|b|) for 3-vectors."""
    a = np.stack([ax, ay, az], 1)
    b = np.stack([bx, by, bz], 1)
    nb = np.linalg.norm(b, axis=1)
    floor = 1e-6 * np.sqrt(np.mean(nb * nb)) + 1e-300
    return np.linalg.norm(a - b, axis=1) / (nb + floor)


def assert_close(name, a, b, tol):
    e = scaled_err(a, b)
    assert np.all(np.isfinite(a)), f"{name}: non-finite values"
    assert e.max() <= tol, f"{name}: max scaled error {e.max():.3e} > {tol:.1e} (median {np.median(e):.2e})"


def assert_vec_close(name, got, ref, tol):
    e = vec_err(*got, *ref)
    assert e.max() <= tol, f"{name}: max scaled error {e.max():.3e} > {tol:.1e} (median {np.median(e):.2e})"


# FP64 GPU (and oracle) against the reference: summation order, fused multiply-add and
# rsqrt/pow implementation differences only.
FP64_TOL = {"h": 1e-12, "rho": 1e-12, "pressure": 1e-12, "sound": 1e-12, "hfactor": 1e-11,
            "invomega": 1e-11, "zeta": 1e-10, "gpot": 1e-11, "div_v": 1e-9, "dudt": 1e-9,
            "a": 1e-10, "ag": 1e-10}


def check_fp64(got: dict, ref: dict, gravity: bool):
    for k in ("h", "rho", "pressure", "sound", "hfactor", "invomega", "zeta", "div_v", "dudt"):
        assert_close(k, got[k], ref[k], FP64_TOL[k])
    assert_vec_close("a", (got["ax"], got["ay"], got["az"]), (ref["ax"], ref["ay"], ref["az"]), FP64_TOL["a"])
    if gravity:
        assert_vec_close("atree", (got["agx"], got["agy"], got["agz"]),
                         (ref["agx"], ref["agy"], ref["agz"]), FP64_TOL["ag"])
        assert_close("gpot", got["gpot"], ref["gpot"], FP64_TOL["gpot"])


def csr_lists(off, ids):
    return [np.sort(ids[off[i]:off[i + 1]]) for i in range(len(off) - 1)]


def same_lists(a, b):
    bad = [i for i, (x, y) in enumerate(zip(a, b)) if not np.array_equal(np.sort(x), np.sort(y))]
    return bad
