"""Generate the golden fixtures from the upstream GANDALF code itself.

Runs oracle/_ref/gsph_ref_harness (the reference compiled from its own sources by
oracle/Makefile.ref) on small seeded particle sets and stores, per case:
  inputs        x y z vx vy vz m u h (the harness input)
  particles     the reference's per-particle results (oracle/refio.PARTICLE_FIELDS order)
  cells         the reference KD-tree cells (oracle/refio.CELL_FIELDS order)
  leaf_*        leaf membership (depth-first leaf id -> sorted input ids, CSR)
  hydro_*       SPH neighbour lists per particle (sorted input ids, CSR)
  direct_*      Newtonian direct-sum partners per particle as (count, hash)
  gcell_*       multipole cells per leaf as (count, hash)
  star_*        (cases with stars) star inputs x y z vx vy vz m h and the reference's
                star <- gas results (oracle/refio.STAR_FIELDS order)
Hashes are sums of splitmix64(id) (gandalf_gb300.sph.list_hash).

KDK cases (multi-step runs of the reference's main loop with block timesteps) store the
inputs, the integrator parameters (kdk_*), the final per-particle state
(oracle/refio.KDK_FIELDS order) and the integer-time globals (oracle/refio.KDK_GLOBAL).

    python tests/golden/make_golden.py     # needs oracle/_ref built
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from gandalf_gb300 import ics as ics_mod  # noqa: E402
from gandalf_gb300.sph import list_hash  # noqa: E402
from oracle import refio  # noqa: E402

CASES = {
    "cube2048": lambda: ics_mod.periodic_cube(2048, seed=11),
    "plummer2048": lambda: ics_mod.plummer_sphere(2048, seed=12),
    "plummer_stars2048": lambda: ics_mod.with_stars(ics_mod.plummer_sphere(2048, seed=13), 16, h=0.05,
                                                    sigma_v=0.1, seed=14),
}


def _cube_adiabatic(n, seed):
    c = ics_mod.periodic_cube(n, seed=seed)
    c["kdk"] = dict(nlevels=3, level_diff_max=1, courant_mult=0.15, accel_mult=0.3, energy_mult=0.4)
    return c


KDK_CASES = {
    "rotating_kdk2048": (lambda: ics_mod.rotating_cloud(2048, seed=41), 8),
    "cube_kdk2048": (lambda: _cube_adiabatic(2048, 42), 6),
}


def make_kdk(name):
    fn, nsteps = KDK_CASES[name]
    c = fn()
    prm = dict(c["params"])
    kdk = dict(c["kdk"])
    kdk["nsteps"] = nsteps
    r = refio.run_kdk(c, prm, kdk)
    out = {k: c[k] for k in ("x", "y", "z", "vx", "vy", "vz", "m", "u", "h")}
    out["state"] = np.stack([r["particles"][k] for k in refio.KDK_FIELDS], axis=1)
    out["global"] = np.array([r["global"][k] for k in refio.KDK_GLOBAL])
    for k, v in prm.items():
        out["param_" + k] = np.asarray(v)
    for k, v in kdk.items():
        out["kdk_" + k] = np.asarray(v)
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), name + ".npz")
    np.savez_compressed(path, **out)
    print(f"{path}: {os.path.getsize(path) / 1024:.0f} KiB")


def csr(lists):
    off = np.zeros(len(lists) + 1, dtype=np.int64)
    for i, l in enumerate(lists):
        off[i + 1] = off[i] + len(l)
    ids = np.concatenate([np.sort(np.asarray(l, dtype=np.int32)) for l in lists]) if len(lists) else np.zeros(0, np.int32)
    return off, ids.astype(np.int32)


def make(name):
    c = CASES[name]()
    prm = dict(c["params"])
    r = refio.run(c, prm)
    out = {k: c[k] for k in ("x", "y", "z", "vx", "vy", "vz", "m", "u", "h")}
    out["particles"] = np.stack([r["particles"][k] for k in refio.PARTICLE_FIELDS], axis=1)
    out["cells"] = np.stack([r["cells"][k] for k in refio.CELL_FIELDS], axis=1)
    out["leaf_cell"] = r["leaf_cell"].astype(np.int32)
    out["leaf_off"], out["leaf_ids"] = csr(r["leaf_members"])
    out["hydro_off"], out["hydro_ids"] = csr(r["hydro_neib"])
    out["direct_count"] = np.array([len(l) for l in r["grav_direct"]], dtype=np.int64)
    out["direct_hash"] = np.array([list_hash(l) for l in r["grav_direct"]], dtype=np.uint64)
    out["gcell_leaf"] = r["gcell_leaf"].astype(np.int32)
    out["gcell_count"] = np.array([len(l) for l in r["gcell_lists"]], dtype=np.int64)
    out["gcell_hash"] = np.array([list_hash(l) for l in r["gcell_lists"]], dtype=np.uint64)
    if c.get("stars") is not None:
        for k in refio.STAR_KEYS:
            out["star_" + k] = c["stars"][k]
        out["star_results"] = np.stack([r["stars"][k] for k in refio.STAR_FIELDS], axis=1)
    for k, v in prm.items():
        out["param_" + k] = np.asarray(v)
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), name + ".npz")
    np.savez_compressed(path, **out)
    print(f"{path}: {os.path.getsize(path) / 1024:.0f} KiB")


if __name__ == "__main__":
    for name in (sys.argv[1:] or list(CASES) + list(KDK_CASES)):
        if name in KDK_CASES:
            make_kdk(name)
        else:
            make(name)
