"""Test infrastructure: run the compiled upstream GANDALF path (oracle/_ref) on a
particle set and read back what it computed.

Only tests and the golden-fixture script use this module.  The binary it drives,
``oracle/_ref/gsph_ref_harness``, is built by ``make -f oracle/Makefile.ref`` from the
upstream sources and exists only where those sources are available.
"""
from __future__ import annotations

import os
import struct
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
HARNESS = os.path.join(HERE, "_ref", "gsph_ref_harness")

PARTICLE_FIELDS = ["h", "rho", "invomega", "zeta", "hfactor", "pressure", "sound", "u",
                   "div_v", "dudt", "ax", "ay", "az", "agx", "agy", "agz", "gpot",
                   "gpot_hydro", "hrangesqd", "levelneib"]
CELL_FIELDS = ["N", "level", "copen", "cnext", "bbmin0", "bbmin1", "bbmin2", "bbmax0",
               "bbmax1", "bbmax2", "hbmin0", "hbmin1", "hbmin2", "hbmax0", "hbmax1",
               "hbmax2", "rcell0", "rcell1", "rcell2", "r0", "r1", "r2", "m", "rmax",
               "hmax", "cdistsqd", "q0", "q1", "q2", "q3", "q4", "maxsound", "Nactive", "id"]

DEFAULTS = dict(self_gravity=0, eos=0, periodic=0, nleafmax=8, multipole=1, h_fac=1.2,
                h_converge=0.01, alpha_visc=1.0, beta_visc=2.0, gamma_eos=5.0 / 3.0,
                thetamaxsqd=0.25, temp0=1.0, mu_bar=1.0, boxmin=(0.0, 0.0, 0.0),
                boxmax=(1.0, 1.0, 1.0))


def available() -> bool:
    return os.path.exists(HARNESS)


STAR_KEYS = ("x", "y", "z", "vx", "vy", "vz", "m", "h")
KDK_FIELDS = ["x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az", "h", "rho", "u", "level", "nstep", "nlast",
              "levelneib", "dt", "tlast", "dudt", "div_v", "gpot", "invomega", "pressure", "sound"]
KDK_GLOBAL = ["n", "t", "timestep", "level_max", "level_step", "nresync", "Nsteps", "dt_max"]
KDK_DEFAULTS = dict(nsteps=1, nlevels=1, level_diff_max=1, courant_mult=0.15, accel_mult=0.3, energy_mult=0.4)
STAR_FIELDS = ["ax", "ay", "az", "adotx", "adoty", "adotz", "gpot"]


def write_input(path: str, ics: dict, params: dict, kdk: dict | None = None) -> None:
    """ics may carry ``stars``: a dict of star arrays (STAR_KEYS); kdk: a multi-step run
    (KDK_DEFAULTS keys)."""
    p = dict(DEFAULTS)
    p.update(params)
    n = len(ics["x"])
    stars = ics.get("stars")
    nstar = 0 if stars is None else len(stars["x"])
    with open(path, "wb") as f:
        f.write(b"GSPHIN01")
        f.write(struct.pack("<8i", n, int(p["self_gravity"]), int(p["eos"]), int(p["periodic"]),
                            int(p["nleafmax"]), int(p["multipole"]), nstar, 1 if kdk else 0))
        f.write(struct.pack("<8d", p["h_fac"], p["h_converge"], p["alpha_visc"], p["beta_visc"],
                            p["gamma_eos"], p["thetamaxsqd"], p["temp0"], p["mu_bar"]))
        f.write(struct.pack("<6d", *p["boxmin"], *p["boxmax"]))
        if kdk:
            k = dict(KDK_DEFAULTS)
            k.update(kdk)
            f.write(struct.pack("<4i", int(k["nsteps"]), int(k["nlevels"]), int(k["level_diff_max"]), 0))
            f.write(struct.pack("<4d", k["courant_mult"], k["accel_mult"], k["energy_mult"], 0.0))
        for key in ("x", "y", "z", "vx", "vy", "vz", "m", "u", "h"):
            f.write(np.ascontiguousarray(ics[key], dtype="<f8").tobytes())
        for key in STAR_KEYS if nstar else ():
            f.write(np.ascontiguousarray(stars[key], dtype="<f8").tobytes())


def _blocks(path, dtype):
    out = []
    with open(path, "rb") as f:
        data = f.read()
    off = 0
    while off < len(data):
        (n,) = struct.unpack_from("<q", data, off)
        off += 8
        a = np.frombuffer(data, dtype=dtype, count=n, offset=off).copy()
        off += n * np.dtype(dtype).itemsize
        out.append(a)
    return out


def _csr(off, ids):
    return [ids[off[i]:off[i + 1]] for i in range(len(off) - 1)]


def run_kdk(ics: dict, params: dict, kdk: dict, workdir: str | None = None) -> dict:
    """SetupSimulation + kdk["nsteps"] reference main-loop steps; per-particle state
    (KDK_FIELDS, input order) and the integer-time globals (KDK_GLOBAL)."""
    if not available():
        raise RuntimeError("upstream harness not built (make -f oracle/Makefile.ref)")
    tmp = os.path.abspath(workdir) if workdir else tempfile.mkdtemp(prefix="gsph_kdk_")
    os.makedirs(tmp, exist_ok=True)
    inp = os.path.join(tmp, "input.bin")
    write_input(inp, ics, params, kdk)
    res = subprocess.run([HARNESS, inp, tmp], capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"reference harness failed ({res.returncode}): {res.stdout[-2000:]}"
                           f"{res.stderr[-2000:]}")
    n = len(ics["x"])
    kb, gb = _blocks(os.path.join(tmp, "kdk.bin"), "<f8")
    kb = kb.reshape(n, len(KDK_FIELDS))
    timing = {}
    with open(os.path.join(tmp, "timing.txt")) as f:
        for line in f:
            k, v = line.split()
            timing[k] = float(v)
    return {"particles": {k: kb[:, i].copy() for i, k in enumerate(KDK_FIELDS)},
            "global": {k: float(gb[i]) for i, k in enumerate(KDK_GLOBAL)}, "timing": timing}


def run(ics: dict, params: dict, workdir: str | None = None) -> dict:
    """Run one reference step; returns particles, cells, leaves, lists and timings."""
    if not available():
        raise RuntimeError("upstream harness not built (make -f oracle/Makefile.ref)")
    tmp = os.path.abspath(workdir) if workdir else tempfile.mkdtemp(prefix="gsph_ref_")
    os.makedirs(tmp, exist_ok=True)
    inp = os.path.join(tmp, "input.bin")
    write_input(inp, ics, params)
    res = subprocess.run([HARNESS, inp, tmp], capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"reference harness failed ({res.returncode}): {res.stdout[-2000:]}"
                           f"{res.stderr[-2000:]}")
    n = len(ics["x"])
    (parts,) = _blocks(os.path.join(tmp, "particles.bin"), "<f8")
    parts = parts.reshape(n, len(PARTICLE_FIELDS))
    (cells,) = _blocks(os.path.join(tmp, "cells.bin"), "<f8")
    cells = cells.reshape(-1, len(CELL_FIELDS))
    leafcell, leafoff, leafpart = _blocks(os.path.join(tmp, "leaves.bin"), "<i4")
    lb = _blocks(os.path.join(tmp, "lists.bin"), "<i4")
    stars = None
    if ics.get("stars") is not None and len(ics["stars"]["x"]):
        (sb,) = _blocks(os.path.join(tmp, "stars.bin"), "<f8")
        sb = sb.reshape(-1, len(STAR_FIELDS))
        stars = {k: sb[:, i].copy() for i, k in enumerate(STAR_FIELDS)}
    timing = {}
    with open(os.path.join(tmp, "timing.txt")) as f:
        for line in f:
            k, v = line.split()
            timing[k] = float(v)
    return {
        "particles": {k: parts[:, i].copy() for i, k in enumerate(PARTICLE_FIELDS)},
        "cells": {k: cells[:, i].copy() for i, k in enumerate(CELL_FIELDS)},
        "leaf_cell": leafcell, "leaf_members": _csr(leafoff, leafpart),
        "hydro_neib": _csr(lb[0], lb[1]), "grav_direct": _csr(lb[2], lb[3]),
        "grav_smooth": _csr(lb[4], lb[5]),
        "gcell_leaf": lb[6], "gcell_lists": _csr(lb[7], lb[8]),
        "timing": timing, "stars": stars,
    }
