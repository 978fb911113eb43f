"""Comparison helpers shared by the parity tests (tolerances are stated per call)."""
from __future__ import annotations

import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
PARTICLE_FIELDS = ["h", "rho", "invomega", "zeta", "hfactor", "pressure", "sound", "u",
                   "div_v", "dudt", "ax", "ay", "az", "agx", "agy", "agz", "gpot",
                   "gpot_hydro", "hrangesqd", "levelneib"]
INPUT_KEYS = ("x", "y", "z", "vx", "vy", "vz", "m", "u", "h")


STAR_KEYS = ("x", "y", "z", "vx", "vy", "vz", "m", "h")
STAR_FIELDS = ["ax", "ay", "az", "adotx", "adoty", "adotz", "gpot"]


def load_golden(name):
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    ics = {k: d[k] for k in INPUT_KEYS}
    if "star_x" in d.files:
        ics["stars"] = {k: d["star_" + k] for k in STAR_KEYS}
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


# Star <- gas results (FP64): summation order and rsqrt/pow differences only.  adot: the
# reference weighs one of its terms with a single-precision powf (NbodyHermite4.cpp:194),
# whose last float bit differs between math libraries.
STAR_TOL = {"a": 1e-12, "adot": 1e-6, "gpot": 1e-12}


def check_stars(got: dict, ref: dict):
    assert_vec_close("star a", (got["ax"], got["ay"], got["az"]), (ref["ax"], ref["ay"], ref["az"]), STAR_TOL["a"])
    assert_vec_close("star adot", (got["adotx"], got["adoty"], got["adotz"]),
                     (ref["adotx"], ref["adoty"], ref["adotz"]), STAR_TOL["adot"])
    assert_close("star gpot", got["gpot"], ref["gpot"], STAR_TOL["gpot"])


def star_results(d):
    return {k: d["star_results"][:, i] for i, k in enumerate(STAR_FIELDS)}


def csr_lists(off, ids):
    return [np.sort(ids[off[i]:off[i + 1]]) for i in range(len(off) - 1)]


def same_lists(a, b):
    bad = [i for i, (x, y) in enumerate(zip(a, b)) if not np.array_equal(np.sort(x), np.sort(y))]
    return bad


def mixed_errors(got: dict, ref: dict) -> dict:
    """Relative errors of the mixed form against fp64: per-particle relative error of
    each scalar (rms and max), and for the acceleration vectors |Δa|/|a| per particle
    plus the normalised rms sqrt(sum |Δa|^2 / sum |a|^2)."""
    out = {}
    for k in ("h", "rho", "pressure", "invomega"):
        if k not in got:
            continue
        e = np.abs(got[k] - ref[k]) / np.abs(ref[k])
        out[k] = (float(np.sqrt(np.mean(e * e))), float(e.max()))
    for name, ks in (("a", ("ax", "ay", "az")), ("ag", ("agx", "agy", "agz"))):
        if ks[0] not in got:
            continue
        A = np.stack([got[k] for k in ks], 1)
        B = np.stack([ref[k] for k in ks], 1)
        nb = np.linalg.norm(B, axis=1)
        if not np.any(nb > 0):
            continue
        d = np.linalg.norm(A - B, axis=1)
        e = d / np.maximum(nb, 1e-300)
        out[name] = (float(np.sqrt(np.mean(e * e))), float(e.max()))
        out[name + "_nrms"] = float(np.sqrt(np.sum(d * d) / np.sum(nb * nb)))
    for k in ("dudt", "gpot", "div_v"):
        if k not in got:
            continue
        b = ref[k]
        if not np.any(b != 0):
            continue
        e = np.abs(got[k] - b) / (np.abs(b) + 1e-3 * np.sqrt(np.mean(b * b)))
        out[k] = (float(np.sqrt(np.mean(e * e))), float(e.max()))
    return out


# Mixed form against fp64: rms and max of the relative errors (mixed_errors).
MIXED_TOL = {"h": (1e-5, 1e-2), "rho": (1e-4, 1e-2), "pressure": (1e-4, 1e-2), "invomega": (1e-4, 1e-2),
             "a": (1e-4, 5e-2), "ag": (1e-4, 5e-2), "a_nrms": 1e-4, "ag_nrms": 1e-4,
             "dudt": (1e-3, 1e-1), "gpot": (1e-5, 1e-3), "div_v": (1e-3, 1e-1)}


def check_mixed(got: dict, ref: dict):
    errs = mixed_errors(got, ref)
    bad = []
    for k, v in errs.items():
        tol = MIXED_TOL[k]
        if isinstance(v, tuple):
            if not (v[0] <= tol[0] and v[1] <= tol[1]):
                bad.append(f"{k}: rms {v[0]:.2e} max {v[1]:.2e} > {tol}")
        elif not v <= tol:
            bad.append(f"{k}: {v:.2e} > {tol}")
    assert not bad, "; ".join(bad) + f" | all: {errs}"
    return errs


def gradh_record_dtype():
    """A record with GradhSphParticle<3>'s field order (src/Headers/Particle.h:133-368)."""
    fields = [("flags", "<u4"), ("ptype", "<i4"), ("iorig", "<i4"), ("sinkid", "<i4"),
              ("levelneib", "<i4"), ("nstep", "<i4"), ("nlast", "<i4"), ("level", "<i4"),
              ("r", "<f8", 3), ("v", "<f8", 3), ("a", "<f8", 3), ("atree", "<f8", 3),
              ("r0", "<f8", 3), ("v0", "<f8", 3), ("a0", "<f8", 3), ("m", "<f8"), ("h", "<f8"),
              ("h_dust", "<f8"), ("hrangesqd", "<f8"), ("hfactor", "<f8"), ("sound", "<f8"),
              ("rho", "<f8"), ("pressure", "<f8"), ("u", "<f8"), ("u0", "<f8"), ("dudt0", "<f8"),
              ("dudt", "<f8"), ("gpot", "<f8"), ("gpot_hydro", "<f8"), ("dt", "<f8"),
              ("dt_next", "<f8"), ("tlast", "<f8"), ("ionfrac", "<f8"), ("Xion", "<f8"),
              ("ueq", "<f8"), ("dt_therm", "<f8"), ("vsig_max", "<f8"), ("rad_pres", "<f8", 3),
              ("ionstate", "<i4"), ("pad", "<i4"), ("div_v", "<f8"), ("alpha", "<f8"),
              ("dalphadt", "<f8"), ("invomega", "<f8"), ("zeta", "<f8")]
    return np.dtype(fields)
