"""Host-side mirror of the reference's SPH neighbour-search interface on the GPU.

``GradhSphTree`` stands in for ``GradhSphTree<3,GradhSphParticle>``
(src/Headers/SphNeighbourSearch.h:173-227): the same calls in the same order —
``BuildTree``, ``UpdateAllSphProperties``, ``UpdateAllSphHydroForces``,
``UpdateAllSphForces`` — backed by the C ABI of libgsph_gb300.so.  Failures raise
``GandalfError``, as the reference's ExceptionHandler does in Python mode
(src/Common/Exception.cpp:49-60).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native

EOS = {"energy_eqn": 0, "isothermal": 1}
MULTIPOLE = {"monopole": 0, "quadrupole": 1}
PRECISION = {"fp64": 0, "mixed": 1}


class GandalfError(RuntimeError):
    """Raised for every failed call (the reference's GandalfError)."""


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def make_config(params: dict | None = None, **kw) -> _native.Config:
    """Config from GANDALF-style parameters (unknown keys are ignored)."""
    lib = _native.load()
    cfg = _native.Config()
    lib.gsph_config_defaults(ctypes.byref(cfg))
    p = dict(params or {})
    p.update(kw)
    if "eos" in p and isinstance(p["eos"], str):
        p["eos"] = EOS[p["eos"]]
    if "gas_eos" in p:
        p["eos"] = EOS[p["gas_eos"]] if isinstance(p["gas_eos"], str) else int(p["gas_eos"])
    if "multipole" in p and isinstance(p["multipole"], str):
        p["multipole"] = MULTIPOLE[p["multipole"]]
    if "precision" in p and isinstance(p["precision"], str):
        p["precision"] = PRECISION[p["precision"]]
    if "Nleafmax" in p:
        p["nleafmax"] = p["Nleafmax"]
    for k in ("ndim", "nleafmax", "hydro_forces", "self_gravity", "eos", "multipole", "periodic", "precision",
              "compensated"):
        if k in p:
            setattr(cfg, k, int(p[k]))
    for k in ("h_fac", "h_converge", "alpha_visc", "beta_visc", "gamma_eos", "temp0", "mu_bar",
              "thetamaxsqd"):
        if k in p:
            setattr(cfg, k, float(p[k]))
    for k in range(3):
        if "boxmin" in p:
            cfg.boxmin[k] = float(p["boxmin"][k])
        if "boxmax" in p:
            cfg.boxmax[k] = float(p["boxmax"][k])
    return cfg


class GradhSphTree:
    """One simulation's particle step on one GPU."""

    def __init__(self, params: dict | None = None, device: int = 0, **kw):
        self._lib = _native.load()
        self.config = make_config(params, **kw)
        self._ctx = self._lib.gsph_create(ctypes.byref(self.config), int(device))
        if not self._ctx:
            code = self._lib.gsph_create_error()
            raise GandalfError(f"gsph_create failed: {_native.ERRORS.get(code, code)}")
        self.n = 0
        self.nstar = 0

    def close(self):
        if getattr(self, "_ctx", None):
            self._lib.gsph_destroy(self._ctx)
            self._ctx = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, rc, what):
        if rc != _native.GSPH_OK:
            msg = self._lib.gsph_last_error(self._ctx)
            raise GandalfError(f"{what}: {_native.ERRORS.get(rc, rc)}: "
                               f"{msg.decode() if msg else ''}")

    # ---- import (Simulation::ImportArraySph) ------------------------------------------
    def set_particles(self, ics: dict):
        """Import x y z vx vy vz m u h from host numpy arrays or CUDA torch tensors."""
        keys = ("x", "y", "z", "vx", "vy", "vz", "m", "u", "h")
        first = ics["x"]
        if hasattr(first, "is_cuda") and first.is_cuda:
            arrs = [ics[k].contiguous().double() for k in keys]
            ptrs = [ctypes.c_void_p(a.data_ptr()) for a in arrs]
            self._keep = arrs
            rc = self._lib.gsph_set_particles_device(self._ctx, len(arrs[0]), *ptrs)
            self.n = len(arrs[0])
        else:
            arrs = [np.ascontiguousarray(ics[k], dtype=np.float64) for k in keys]
            rc = self._lib.gsph_set_particles(self._ctx, len(arrs[0]), *[_dp(a) for a in arrs])
            self.n = len(arrs[0])
        self._check(rc, "set_particles")
        if ics.get("stars") is not None:
            self.set_stars(ics["stars"])

    # ---- star particles (Simulation::ImportArrayNbody) ---------------------------------
    STAR_KEYS = ("x", "y", "z", "vx", "vy", "vz", "m", "h")
    STAR_FIELDS = ("ax", "ay", "az", "adotx", "adoty", "adotz", "gpot")

    def set_stars(self, stars: dict | None):
        """Star particles x y z vx vy vz m h (host arrays); None or empty removes them."""
        if stars is None or len(stars["x"]) == 0:
            self._check(self._lib.gsph_set_stars(self._ctx, 0, *([None] * 8)), "set_stars")
            self.nstar = 0
            return
        arrs = [np.ascontiguousarray(stars[k], dtype=np.float64) for k in self.STAR_KEYS]
        self._check(self._lib.gsph_set_stars(self._ctx, len(arrs[0]), *[_dp(a) for a in arrs]), "set_stars")
        self.nstar = len(arrs[0])

    def UpdateAllStarGasForces(self):
        self._check(self._lib.gsph_update_all_star_gas_forces(self._ctx), "UpdateAllStarGasForces")

    def star_forces(self) -> dict:
        """Gas <- star results of the last star pass: a, adot, gpot per star."""
        outs = [np.zeros(self.nstar) for _ in self.STAR_FIELDS]
        self._check(self._lib.gsph_get_star_forces(self._ctx, *[_dp(a) for a in outs]), "star_forces")
        return dict(zip(self.STAR_FIELDS, outs))

    def set_particles_aos(self, records: np.ndarray, offsets: dict):
        """Import a structured array of particle records (byte offsets per field)."""
        off = _native.FieldOffsets(**{k: int(offsets.get(k, -1)) for k, _ in _native.FieldOffsets._fields_})
        rc = self._lib.gsph_set_particles_aos(self._ctx, records.ctypes.data, len(records),
                                              records.dtype.itemsize, ctypes.byref(off))
        self.n = len(records)
        self._check(rc, "set_particles_aos")

    def get_particles_aos(self, records: np.ndarray, offsets: dict):
        """Write the computed output fields into the records (only those; with a flags
        offset only the active particles', plus levelneib of every particle)."""
        off = _native.FieldOffsets(**{k: int(offsets.get(k, -1)) for k, _ in _native.FieldOffsets._fields_})
        rc = self._lib.gsph_get_particles_aos(self._ctx, records.ctypes.data, len(records),
                                              records.dtype.itemsize, ctypes.byref(off))
        self._check(rc, "get_particles_aos")

    def UpdateActiveParticleCounters(self, records: np.ndarray, offsets: dict):
        """Re-read the records' flags and levels into the current tree (no rebuild)."""
        off = _native.FieldOffsets(**{k: int(offsets.get(k, -1)) for k, _ in _native.FieldOffsets._fields_})
        rc = self._lib.gsph_update_active_particle_counters(self._ctx, records.ctypes.data, len(records),
                                                            records.dtype.itemsize, ctypes.byref(off))
        self._check(rc, "UpdateActiveParticleCounters")

    def GetMaximumSmoothingLength(self) -> float:
        out = ctypes.c_double()
        self._check(self._lib.gsph_get_maximum_smoothing_length(self._ctx, ctypes.byref(out)),
                    "GetMaximumSmoothingLength")
        return out.value

    # ---- the reference's virtual interface ----------------------------------------------
    def BuildTree(self):
        self._check(self._lib.gsph_build_tree(self._ctx), "BuildTree")

    def UpdateAllSphProperties(self):
        self._check(self._lib.gsph_update_all_sph_properties(self._ctx), "UpdateAllSphProperties")

    def UpdateAllSphHydroForces(self):
        self._check(self._lib.gsph_update_all_sph_hydro_forces(self._ctx), "UpdateAllSphHydroForces")

    def UpdateAllSphForces(self):
        self._check(self._lib.gsph_update_all_sph_forces(self._ctx), "UpdateAllSphForces")

    def step(self, graph: bool = False):
        """BuildTree + UpdateAllSphProperties + the configured force pass (graph=True:
        replayed from a captured CUDA graph)."""
        if graph:
            self._check(self._lib.gsph_step_graph(self._ctx), "step_graph")
        else:
            self._check(self._lib.gsph_step(self._ctx), "step")

    build_tree = BuildTree
    update_all_sph_properties = UpdateAllSphProperties
    update_all_sph_hydro_forces = UpdateAllSphHydroForces
    update_all_sph_forces = UpdateAllSphForces
    update_all_star_gas_forces = UpdateAllStarGasForces

    # ---- KDK integration with block timesteps (SphSimulation::MainLoop) -------------------
    def kdk_setup(self, **kw):
        """PostInitialConditionsSetup: nlevels, level_diff_max, courant_mult, accel_mult,
        energy_mult as the reference's parameters."""
        k = _native.KdkConfig()
        self._lib.gsph_kdk_config_defaults(ctypes.byref(k))
        for name, val in kw.items():
            setattr(k, name, type(getattr(k, name))(val))
        self._check(self._lib.gsph_kdk_setup(self._ctx, ctypes.byref(k)), "kdk_setup")

    def kdk_steps(self, nsteps: int, graph: bool = True):
        self._check(self._lib.gsph_kdk_steps(self._ctx, int(nsteps), int(graph)), "kdk_steps")

    def kdk_status(self) -> dict:
        st = _native.KdkStatus()
        self._check(self._lib.gsph_kdk_get_status(self._ctx, ctypes.byref(st)), "kdk_status")
        return {k: getattr(st, k) for k, _ in _native.KdkStatus._fields_}

    def kdk_timing(self) -> dict:
        st = _native.KdkTiming()
        self._check(self._lib.gsph_kdk_get_timing(self._ctx, ctypes.byref(st)), "kdk_timing")
        return {k: getattr(st, k) for k, _ in _native.KdkTiming._fields_}

    def kdk_state(self, name: str, out: np.ndarray | None = None) -> np.ndarray:
        """One integration field (input order); ``out``: an n-double array to fill."""
        if out is None:
            out = np.empty(self.n, dtype=np.float64)
        self._check(self._lib.gsph_kdk_get_state(self._ctx, _native.KDK_FIELDS.index(name), _dp(out)), "kdk_state")
        return out

    # ---- results --------------------------------------------------------------------------
    def field(self, name: str, out: np.ndarray | None = None) -> np.ndarray:
        """One result field (input order); ``out``: an n-double array to fill."""
        if out is None:
            out = np.empty(self.n, dtype=np.float64)
        self._check(self._lib.gsph_get_field(self._ctx, _native.FIELD_ID[name], _dp(out)), "get_field")
        return out

    def field_device(self, name: str, out_ptr: int):
        self._check(self._lib.gsph_get_field_device(self._ctx, _native.FIELD_ID[name],
                                                    ctypes.c_void_p(out_ptr)), "get_field_device")

    def results(self) -> dict:
        return {k: self.field(k) for k in _native.FIELDS}

    def stats(self) -> dict:
        s = _native.Stats()
        self._check(self._lib.gsph_get_stats(self._ctx, ctypes.byref(s)), "get_stats")
        return {k: getattr(s, k) for k, _ in _native.Stats._fields_}

    # ---- autotuning (gsph_autotune) -------------------------------------------------------
    def tuning(self) -> dict:
        t = _native.Tuning()
        self._check(self._lib.gsph_get_tuning(self._ctx, ctypes.byref(t)), "get_tuning")
        return {k: getattr(t, k) for k, _ in _native.Tuning._fields_}

    def set_tuning(self, **kw):
        t = _native.Tuning(**{**self.tuning(), **kw})
        self._check(self._lib.gsph_set_tuning(self._ctx, ctypes.byref(t)), "set_tuning")

    def autotune(self, steps: int = 2) -> dict:
        """Leaf size, warps per cell (near-list depth before the 8-warp kernel) and list tile
        depths chosen by timing the imported particles' step; the best is applied."""
        best = _native.Tuning()
        cap = 32
        tried = (_native.Tuning * cap)()
        ms = (ctypes.c_double * cap)()
        nt = ctypes.c_int32()
        self._check(self._lib.gsph_autotune(self._ctx, int(steps), ctypes.byref(best), tried, ms, cap,
                                            ctypes.byref(nt)), "autotune")
        fields = [k for k, _ in _native.Tuning._fields_]
        return {**{k: getattr(best, k) for k in fields},
                "tried": [dict({k: getattr(tried[i], k) for k in fields}, ms_per_step=ms[i])
                          for i in range(min(nt.value, cap))]}

    def set_stream(self, stream_ptr: int | None):
        """Run on the given cudaStream_t (e.g. torch.cuda.current_stream().cuda_stream)."""
        self._check(self._lib.gsph_set_stream(self._ctx, ctypes.c_void_p(stream_ptr or 0)), "set_stream")

    # ---- verification ---------------------------------------------------------------------
    def set_recording(self, enable: bool, max_sph: int = 512):
        self._check(self._lib.gsph_set_recording(self._ctx, int(enable), int(max_sph)), "set_recording")

    def sph_neighbours(self) -> list:
        tot = self._lib.gsph_get_sph_neighbours(self._ctx, None, None)
        if tot < 0:
            self._check(int(tot), "sph_neighbours")
        off = np.zeros(self.n + 1, dtype=np.int64)
        ids = np.zeros(max(int(tot), 1), dtype=np.int32)
        r = self._lib.gsph_get_sph_neighbours(self._ctx, off.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                                              ids.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)))
        if r < 0:
            self._check(int(r), "sph_neighbours")
        return [ids[off[i]:off[i + 1]] for i in range(self.n)]

    def sph_neighbours_csr(self):
        """The recorded SPH neighbour lists as CSR arrays (offsets n+1, input ids)."""
        tot = self._lib.gsph_get_sph_neighbours(self._ctx, None, None)
        if tot < 0:
            self._check(int(tot), "sph_neighbours")
        off = np.zeros(self.n + 1, dtype=np.int64)
        ids = np.zeros(max(int(tot), 1), dtype=np.int32)
        r = self._lib.gsph_get_sph_neighbours(self._ctx, off.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                                              ids.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)))
        if r < 0:
            self._check(int(r), "sph_neighbours")
        return off, ids[:int(tot)]

    def set_list_recording(self, max_direct: int, max_cells: int):
        self._check(self._lib.gsph_set_list_recording(self._ctx, int(max_direct), int(max_cells)),
                    "set_list_recording")

    def _csr(self, fn, count):
        tot = fn(self._ctx, None, None)
        if tot < 0:
            self._check(int(tot), "lists")
        off = np.zeros(count + 1, dtype=np.int64)
        ids = np.zeros(max(int(tot), 1), dtype=np.int32)
        r = fn(self._ctx, off.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
               ids.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)))
        if r < 0:
            self._check(int(r), "lists")
        return [ids[off[i]:off[i + 1]] for i in range(count)]

    def direct_lists(self) -> list:
        """Direct-sum partners (input ids) of every particle, input order."""
        return self._csr(self._lib.gsph_get_direct_lists, self.n)

    def cell_lists(self) -> list:
        """Multipole cells (depth-first ids) of every leaf, in cell_summary's leaf order."""
        return self._csr(self._lib.gsph_get_cell_lists, int(self.stats()["nleaf"]))

    def direct_summary(self):
        cnt = np.zeros(self.n, dtype=np.int64)
        hsh = np.zeros(self.n, dtype=np.uint64)
        self._check(self._lib.gsph_get_direct_summary(self._ctx, cnt.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                                                      hsh.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64))),
                    "direct_summary")
        return cnt, hsh

    def cell_summary(self):
        st = self.stats()
        nl = int(st["nleaf"])
        leaf = np.zeros(nl, dtype=np.int32)
        cnt = np.zeros(nl, dtype=np.int64)
        hsh = np.zeros(nl, dtype=np.uint64)
        self._check(self._lib.gsph_get_cell_summary(self._ctx, leaf.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                                    cnt.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)),
                                                    hsh.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64))),
                    "cell_summary")
        return leaf, cnt, hsh

    def tree(self) -> dict:
        st = self.stats()
        nc = int(st["ncell"])
        cn = np.zeros(nc, dtype=np.int32)
        cf = np.zeros(nc, dtype=np.int32)
        order = np.zeros(self.n, dtype=np.int32)
        data = np.zeros((nc, 31), dtype=np.float64)
        P = ctypes.POINTER(ctypes.c_int32)
        self._check(self._lib.gsph_get_tree(self._ctx, cn.ctypes.data_as(P), cf.ctypes.data_as(P),
                                            order.ctypes.data_as(P), _dp(data)), "get_tree")
        return {"cell_n": cn, "cell_first": cf, "order": order, "cells": data, "ltot": int(st["ltot"])}


def mix64(ids: np.ndarray) -> np.ndarray:
    """The order-independent hash term the kernels sum per list entry (splitmix64)."""
    x = ids.astype(np.uint64) + np.uint64(0x9E3779B97F4A7C15)
    with np.errstate(over="ignore"):
        x = (x ^ (x >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        x = (x ^ (x >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return x ^ (x >> np.uint64(31))


def list_hash(ids) -> np.uint64:
    ids = np.asarray(ids)
    if ids.size == 0:
        return np.uint64(0)
    with np.errstate(over="ignore"):
        return np.sum(mix64(ids), dtype=np.uint64)


class GradhSphBatch:
    """Many independent simulations (mixed-precision GradhSphTree objects) stepped together:
    one persistent launch per pass over all their leaf cells, replayed from one CUDA graph."""

    def __init__(self, trees: list):
        self._lib = _native.load()
        self.trees = list(trees)
        arr = (ctypes.c_void_p * len(self.trees))(*[t._ctx for t in self.trees])
        self._b = self._lib.gsph_batch_create(arr, len(self.trees))
        if not self._b:
            code = self._lib.gsph_create_error()
            raise GandalfError(f"gsph_batch_create failed: {_native.ERRORS.get(code, code)}")

    def step(self):
        rc = self._lib.gsph_batch_step(self._b)
        if rc != _native.GSPH_OK:
            msg = self._lib.gsph_batch_last_error(self._b)
            raise GandalfError(f"batch step: {_native.ERRORS.get(rc, rc)}: {msg.decode() if msg else ''}")

    def stats(self) -> dict:
        ms = ctypes.c_float()
        nl = ctypes.c_int32()
        self._lib.gsph_batch_stats(self._b, ctypes.byref(ms), ctypes.byref(nl))
        return {"ms": ms.value, "launches": nl.value}

    def close(self):
        if getattr(self, "_b", None):
            self._lib.gsph_batch_destroy(self._b)
            self._b = None

    def __del__(self):
        self.close()
