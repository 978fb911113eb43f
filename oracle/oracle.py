"""ORACLE — test infrastructure, not product code.

ctypes front end of ``oracle/gsph_oracle.cpp``, the CPU restatement of GANDALF's grad-h
SPH + KD-tree gravity step.  Only tests/, ``__graft_entry__.smoke()`` and bench.py's
CPU-baseline leg import this module, and only as the checker.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "gsph_oracle.cpp")
BUILD_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD_DIR, "libgsph_oracle.so")

PARTICLE_FIELDS = ["h", "rho", "invomega", "zeta", "hfactor", "pressure", "sound", "u",
                   "div_v", "dudt", "ax", "ay", "az", "agx", "agy", "agz", "gpot",
                   "gpot_hydro", "hrangesqd", "levelneib"]
STAR_KEYS = ("x", "y", "z", "vx", "vy", "vz", "m", "h")
STAR_FIELDS = ["ax", "ay", "az", "adotx", "adoty", "adotz", "gpot"]
CELL_FIELDS = ["N", "level", "m", "rmax", "hmax", "cdistsqd", "bbmin0", "bbmin1", "bbmin2",
               "bbmax0", "bbmax1", "bbmax2", "hbmin0", "hbmin1", "hbmin2", "hbmax0", "hbmax1",
               "hbmax2", "rcell0", "rcell1", "rcell2", "r0", "r1", "r2", "q0", "q1", "q2", "q3",
               "q4", "first", "pad"]


class Params(ctypes.Structure):
    _fields_ = [("self_gravity", ctypes.c_int32), ("eos", ctypes.c_int32),
                ("periodic", ctypes.c_int32), ("nleafmax", ctypes.c_int32),
                ("multipole", ctypes.c_int32), ("hydro_forces", ctypes.c_int32),
                ("pad0", ctypes.c_int32), ("pad1", ctypes.c_int32),
                ("h_fac", ctypes.c_double), ("h_converge", ctypes.c_double),
                ("alpha_visc", ctypes.c_double), ("beta_visc", ctypes.c_double),
                ("gamma_eos", ctypes.c_double), ("thetamaxsqd", ctypes.c_double),
                ("temp0", ctypes.c_double), ("mu_bar", ctypes.c_double),
                ("boxmin", ctypes.c_double * 3), ("boxmax", ctypes.c_double * 3)]


DEFAULTS = dict(self_gravity=0, eos=0, periodic=0, nleafmax=8, multipole=1, h_fac=1.2,
                h_converge=0.01, alpha_visc=1.0, beta_visc=2.0, gamma_eos=5.0 / 3.0,
                thetamaxsqd=0.25, temp0=1.0, mu_bar=1.0, boxmin=(0.0, 0.0, 0.0),
                boxmax=(1.0, 1.0, 1.0))


def build(force: bool = False) -> str:
    """Compile the restatement (g++, OpenMP, no FP contraction) into oracle/_build."""
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    os.makedirs(BUILD_DIR, exist_ok=True)
    tmp = LIB + ".tmp"
    cmd = ["g++", "-O3", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-std=c++17",
           SRC, "-o", tmp]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


_lib = None


def _load():
    global _lib
    if _lib is None:
        build()
        lib = ctypes.CDLL(LIB)
        vp, i64, i32, dp = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int, ctypes.POINTER(ctypes.c_double)
        lib.gsph_oracle_create.restype = vp
        lib.gsph_oracle_create.argtypes = [ctypes.POINTER(Params)]
        lib.gsph_oracle_destroy.argtypes = [vp]
        lib.gsph_oracle_run.restype = i32
        lib.gsph_oracle_run.argtypes = [vp, i64] + [dp] * 9 + [i32, i32]
        lib.gsph_oracle_particles.argtypes = [vp, dp]
        lib.gsph_oracle_ncell.restype = i32
        lib.gsph_oracle_ncell.argtypes = [vp]
        lib.gsph_oracle_ltot.restype = i32
        lib.gsph_oracle_ltot.argtypes = [vp]
        lib.gsph_oracle_cells.argtypes = [vp, dp]
        lib.gsph_oracle_order.argtypes = [vp, ctypes.POINTER(ctypes.c_int32)]
        lib.gsph_oracle_list.restype = i64
        lib.gsph_oracle_list.argtypes = [vp, i32, ctypes.POINTER(ctypes.c_int32),
                                         ctypes.POINTER(ctypes.c_int32)]
        lib.gsph_oracle_counts.argtypes = [vp, ctypes.POINTER(ctypes.c_int64)]
        lib.gsph_oracle_summary.argtypes = [vp, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_uint64),
                                            ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int64),
                                            ctypes.POINTER(ctypes.c_uint64)]
        lib.gsph_oracle_run_given.restype = i32
        lib.gsph_oracle_run_given.argtypes = [vp, i64] + [dp] * 15 + [i32, i32]
        lib.gsph_oracle_nleaf.restype = i32
        lib.gsph_oracle_nleaf.argtypes = [vp]
        u8p, i32p = ctypes.POINTER(ctypes.c_uint8), ctypes.POINTER(ctypes.c_int32)
        lib.gsph_oracle_run_active.restype = i32
        lib.gsph_oracle_run_active.argtypes = [vp, i64] + [dp] * 9 + [u8p, i32p, i32p, dp, i32, i32]
        lib.gsph_oracle_levelneib.argtypes = [vp, i32p]
        lib.gsph_oracle_kdk.restype = i32
        lib.gsph_oracle_kdk.argtypes = [vp, i64] + [dp] * 10 + [i32, i32, dp, dp, dp]
        lib.gsph_oracle_set_stars.argtypes = [vp, i32] + [dp] * 8
        lib.gsph_oracle_stars.argtypes = [vp, dp]
        _lib = lib
    return _lib


def make_params(params: dict) -> Params:
    p = dict(DEFAULTS)
    p.update({k: v for k, v in params.items() if k in DEFAULTS})
    s = Params()
    for k in ("self_gravity", "eos", "periodic", "nleafmax", "multipole"):
        setattr(s, k, int(p[k]))
    s.hydro_forces = 1
    for k in ("h_fac", "h_converge", "alpha_visc", "beta_visc", "gamma_eos", "thetamaxsqd",
              "temp0", "mu_bar"):
        setattr(s, k, float(p[k]))
    for k in range(3):
        s.boxmin[k] = float(p["boxmin"][k])
        s.boxmax[k] = float(p["boxmax"][k])
    return s


def _ptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def run(ics: dict, params: dict, lists: bool = False, nthreads: int = 0, summary: bool = False,
        given: dict | None = None) -> dict:
    """One step of the restated algorithm; same result layout as oracle/refio.run.

    lists: full interaction lists (small N only); summary: SPH lists plus (count, hash)
    of direct partners per particle and multipole cells per leaf.  given: the h solve's
    results (h rho invomega zeta pressure sound, input order) to use instead of solving
    — the force pass and its lists for exactly those smoothing lengths.
    """
    lib = _load()
    prm = make_params(params)
    h = lib.gsph_oracle_create(ctypes.byref(prm))
    try:
        stars = ics.get("stars")
        ns = 0 if stars is None else len(stars["x"])
        if ns:
            sarr = [np.ascontiguousarray(stars[k], dtype=np.float64) for k in STAR_KEYS]
            lib.gsph_oracle_set_stars(h, ns, *[_ptr(a) for a in sarr])
        arrs = [np.ascontiguousarray(ics[k], dtype=np.float64)
                for k in ("x", "y", "z", "vx", "vy", "vz", "m", "u", "h")]
        n = len(arrs[0])
        mode = 1 if lists else (2 if summary else 0)
        if given is None:
            st = lib.gsph_oracle_run(h, n, *[_ptr(a) for a in arrs], mode, int(nthreads))
        else:
            gv = [np.ascontiguousarray(given[k], dtype=np.float64)
                  for k in ("h", "rho", "invomega", "zeta", "pressure", "sound")]
            st = lib.gsph_oracle_run_given(h, n, *[_ptr(a) for a in arrs], *[_ptr(a) for a in gv], mode,
                                           int(nthreads))
        if st != 0:
            raise RuntimeError(f"oracle step failed with status {st}")
        out = np.empty((n, len(PARTICLE_FIELDS)))
        lib.gsph_oracle_particles(h, _ptr(out))
        nc = lib.gsph_oracle_ncell(h)
        cells = np.empty((nc, len(CELL_FIELDS)))
        lib.gsph_oracle_cells(h, _ptr(cells))
        order = np.empty(n, dtype=np.int32)
        lib.gsph_oracle_order(h, order.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)))
        counts = (ctypes.c_int64 * 4)()
        lib.gsph_oracle_counts(h, counts)
        star_res = None
        if ns:
            so = np.empty((ns, len(STAR_FIELDS)))
            lib.gsph_oracle_stars(h, _ptr(so))
            star_res = {k: so[:, i].copy() for i, k in enumerate(STAR_FIELDS)}
        res = {
            "stars": star_res,
            "particles": {k: out[:, i].copy() for i, k in enumerate(PARTICLE_FIELDS)},
            "cells": {k: cells[:, i].copy() for i, k in enumerate(CELL_FIELDS)},
            "order": order, "ltot": lib.gsph_oracle_ltot(h),
            "counts": dict(density_pairs=counts[0], hydro_pairs=counts[1],
                           direct_pairs=counts[2], cell_pairs=counts[3]),
        }
        if summary:
            tot = lib.gsph_oracle_list(h, 0, None, None)
            off = np.zeros(n + 1, dtype=np.int32)
            ids = np.zeros(max(tot, 1), dtype=np.int32)
            lib.gsph_oracle_list(h, 0, off.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                 ids.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)))
            res["hydro_neib"] = [ids[off[i]:off[i + 1]] for i in range(n)]
            nl = lib.gsph_oracle_nleaf(h)
            dc = np.zeros(n, dtype=np.int64)
            dh = np.zeros(n, dtype=np.uint64)
            lc = np.zeros(nl, dtype=np.int32)
            cc = np.zeros(nl, dtype=np.int64)
            ch = np.zeros(nl, dtype=np.uint64)
            P64, PU, P32 = ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_int32)
            lib.gsph_oracle_summary(h, dc.ctypes.data_as(P64), dh.ctypes.data_as(PU), lc.ctypes.data_as(P32),
                                    cc.ctypes.data_as(P64), ch.ctypes.data_as(PU))
            res.update(direct_count=dc, direct_hash=dh, leaf_cell=lc, cell_count=cc, cell_hash=ch)
        if lists:
            names = {0: "hydro_neib", 1: "grav_direct", 2: "gcell_lists"}
            for which, name in names.items():
                cnt = n if which < 2 else lib.gsph_oracle_list(h, 3, None, None)
                tot = lib.gsph_oracle_list(h, which, None, None)
                off = np.zeros(cnt + 1, dtype=np.int32)
                ids = np.zeros(max(tot, 1), dtype=np.int32)
                lib.gsph_oracle_list(h, which, off.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                     ids.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)))
                res[name] = [ids[off[i]:off[i + 1]] for i in range(cnt)]
            nl = lib.gsph_oracle_list(h, 3, None, None)
            leaf = np.zeros(max(nl, 1), dtype=np.int32)
            lib.gsph_oracle_list(h, 3, None, leaf.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)))
            res["gcell_leaf"] = leaf[:nl]
        return res
    finally:
        lib.gsph_oracle_destroy(h)


KDK_FIELDS = ["x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az", "h", "rho", "u", "level", "nstep", "nlast",
              "levelneib", "dt", "tlast", "dudt", "div_v", "gpot", "invomega", "pressure", "sound"]
KDK_GLOBAL = ["n", "t", "timestep", "level_max", "level_step", "nresync", "Nsteps", "dt_max"]


def kdk(ics: dict, params: dict, kdk_params: dict, nsteps: int, nthreads: int = 0) -> dict:
    """Setup plus nsteps main-loop steps of the KDK leapfrog with block timesteps.

    Returns the final per-particle state (KDK_FIELDS, input order), the integer-time
    state (KDK_GLOBAL) and timing: setup and step wall seconds, active particle updates
    of the setup and of the steps.
    """
    lib = _load()
    prm = make_params(params)
    hnd = lib.gsph_oracle_create(ctypes.byref(prm))
    try:
        arrs = [np.ascontiguousarray(ics[k], dtype=np.float64)
                for k in ("x", "y", "z", "vx", "vy", "vz", "m", "u", "h")]
        n = len(arrs[0])
        kp = np.array([kdk_params.get("nlevels", 1), kdk_params.get("level_diff_max", 1),
                       kdk_params.get("courant_mult", 0.15), kdk_params.get("accel_mult", 0.3),
                       kdk_params.get("energy_mult", 0.4)], dtype=np.float64)
        state = np.empty((n, len(KDK_FIELDS)))
        glob = np.empty(len(KDK_GLOBAL))
        info = np.zeros(5)
        st = lib.gsph_oracle_kdk(hnd, n, *[_ptr(a) for a in arrs], _ptr(kp), int(nsteps), int(nthreads),
                                 _ptr(state), _ptr(glob), _ptr(info))
        if st != 0:
            raise RuntimeError(f"oracle KDK run failed with status {st}")
        return {"state": {k: state[:, i].copy() for i, k in enumerate(KDK_FIELDS)},
                "global": {k: float(glob[i]) for i, k in enumerate(KDK_GLOBAL)},
                "setup_s": float(info[0]), "steps_s": float(info[1]),
                "setup_updates": int(info[2]), "step_updates": int(info[3]), "status": int(info[4])}
    finally:
        lib.gsph_oracle_destroy(hnd)


STATE_FIELDS = ("rho", "invomega", "zeta", "hfactor", "hrangesqd", "pressure", "sound")


class ActivePasses:
    """Passes with block-timestep semantics on one oracle instance (the tree persists
    between calls, so a repeated pass can reuse it as the reference's main loop does)."""

    def __init__(self, params: dict, nthreads: int = 0):
        self.lib = _load()
        self.prm = make_params(params)
        self.h = self.lib.gsph_oracle_create(ctypes.byref(self.prm))
        self.nthreads = nthreads

    def run(self, ics: dict, active, level, levelneib, state: dict, rebuild: bool = True) -> dict:
        """ics: x y z vx vy vz m u h; state: STATE_FIELDS of every particle (the inactive
        ones keep them).  Returns the per-particle results, levelneib included."""
        arrs = [np.ascontiguousarray(ics[k], dtype=np.float64)
                for k in ("x", "y", "z", "vx", "vy", "vz", "m", "u", "h")]
        n = len(arrs[0])
        act = np.ascontiguousarray(active, dtype=np.uint8)
        lv = np.ascontiguousarray(level, dtype=np.int32)
        lvn = np.ascontiguousarray(levelneib, dtype=np.int32)
        st = np.ascontiguousarray(np.stack([np.asarray(state[k], dtype=np.float64) for k in STATE_FIELDS], 1))
        rc = self.lib.gsph_oracle_run_active(self.h, n, *[_ptr(a) for a in arrs],
                                             act.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)),
                                             lv.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                             lvn.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                             _ptr(st), int(rebuild), int(self.nthreads))
        if rc != 0:
            raise RuntimeError(f"oracle pass failed with status {rc}")
        out = np.empty((n, len(PARTICLE_FIELDS)))
        self.lib.gsph_oracle_particles(self.h, _ptr(out))
        res = {k: out[:, i].copy() for i, k in enumerate(PARTICLE_FIELDS)}
        lvo = np.empty(n, dtype=np.int32)
        self.lib.gsph_oracle_levelneib(self.h, lvo.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)))
        res["levelneib"] = lvo
        return res

    def close(self):
        if self.h:
            self.lib.gsph_oracle_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()
