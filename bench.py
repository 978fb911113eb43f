"""Benchmark: particle updates/s of the grad-h SPH + KD-tree gravity path on one GB300.

Workload (default): the rotating isothermal cloud, N = 1,048,576 gas particles (uniform
sphere R = M = G = 1, m = 2 density perturbation, solid-body rotation with E_rot/|E_grav| =
0.16, E_therm/|E_grav| = 0.26), self-gravity with theta = 0.5 (thetamaxsqd = 0.25) and
quadrupole cells, Nleafmax = 8, 4 block-timestep levels: K steps of the KDK leapfrog main
loop (default K = 20) replayed from one CUDA graph, in the FP64 and the mixed form.  The
unit of work is one active particle through one h solve and one force pass (each KDK
substep counts its active particles, repeats included); seeded synthetic inputs
(gandalf_gb300.ics.rotating_cloud).  Other workloads: --workload plummer_sphere (one full
step of the 262,144-particle Plummer sphere), evrard_sphere (8,388,608 + 64 stars),
kh_ensemble (64 periodic boxes, batched), periodic_cube.

Arms:
  --impl gsph (default)  the CUDA library; `value` is device-resident throughput of the
                         mixed form; `e2e` goes through the C ABI with pinned host arrays
                         copied in and results copied out.
  --impl reference       the CPU restatement of the reference algorithm (oracle/) on all
                         host cores, on the same workload: the same K main-loop steps after
                         the same setup for the rotating cloud.
Under torchrun each rank runs an independent replica on its own GPU (the step has no
exchange between simulations); rank 0 prints the line.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle updates/s (SPH+tree gravity), mixed vs FP64 GPU at ≤1e-4 RMS rel error"
UNIT = "particle updates/s"

# Algorithmic floating-point operations per interaction, counted line by line from the
# reference formulas as written (add, sub, mul, div, sqrt = 1; a multiply-add = 2), the
# unconditional operations only: the artificial-viscosity branch of the hydro pairs (about
# 20 more for approaching pairs) is not counted.
#   density pair, per h iteration   GradhSph.cpp:197-204 (w0, womega, wzeta of one s)     45
#   hydro pair                      GradhSph.cpp:384-447                                  60
#   hydro + softened-gravity pair   GradhSph.cpp:498-571                                 127
#   Newtonian direct term           GradhSph.cpp:671-686                                  24
#   quadrupole cell term            NeighbourSearch.h:423-449                             80
#   monopole cell term              NeighbourSearch.h:359-373                             23
FLOPS = dict(density=45, hydro=60, hydro_grav=127, direct=24, quad=80, mono=23)

# DRAM bytes (read + write) of one force pass of the mixed form, from one-pass ncu captures
# of the force kernels (summed over the kernels of a pass); None where no capture exists.
FORCE_TRAFFIC = {
    ("plummer_sphere", 262144, "mixed"): {"bytes": 45.65e6 + 0.55e6 + 5.15e6,
                                          "source": "profiles/forces_density_mixed_plummer262k_dram.md"},
    # the warp-per-leaf force kernel of a KDK first pass, cold L2 (ncu flushes caches), mean
    # of three launches
    ("rotating_cloud", 1048576, "mixed"): {"bytes": 244.0e6,
                                           "source": "profiles/forces_mixed_rotating_cloud1m_dram.md"},
}


def max_over_ranks(ms, world, device="cuda"):
    """The job's time for replicas on several GPUs: the slowest rank's (all-reduce MAX)."""
    if world <= 1:
        return ms
    import torch
    import torch.distributed as dist
    tt = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    return float(tt.item())


def job_throughput(units_per_rank, ms, world):
    """Whole-job units per second: every rank processes units_per_rank in (at most) ms."""
    return world * units_per_rank / (ms * 1e-3)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=0,
                    help="timed steps (default: 20 KDK steps for rotating_cloud, 3 for evrard_sphere, else 10)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gsph", choices=["gsph", "reference"])
    ap.add_argument("--workload", default="rotating_cloud",
                    choices=["rotating_cloud", "plummer_sphere", "periodic_cube", "evrard_sphere", "kh_ensemble"])
    ap.add_argument("--n", type=int, default=0)
    ap.add_argument("--nleafmax", type=int, default=0,
                    help="evrard_sphere: leaf size to use instead of the autotuner's choice")
    ap.add_argument("--precision", default="auto", choices=["auto", "fp64", "mixed", "mixed_compensated"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-precision", action="store_true",
                    help="rotating_cloud: skip the one-step precision and list comparison of the forms")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-graph", action="store_true", help="launch each step's kernels on the stream "
                    "instead of replaying the captured CUDA graph")
    args = ap.parse_args()
    if not args.steps:
        args.steps = {"rotating_cloud": 20, "evrard_sphere": 3}.get(args.workload, 10)
    return args


def ensemble_main(args, rank, world, local):
    """64 periodic KH boxes of log-uniform N (4,096..131,072), hydro only, mixed form:
    one batched step (persistent launches over all boxes' leaf cells, one CUDA graph)
    against the same 64 simulations stepped one after another (each from its own graph)."""
    import torch
    from gandalf_gb300 import ics as ics_mod
    from gandalf_gb300 import _native
    from gandalf_gb300 import build as gbuild
    from gandalf_gb300.sph import GradhSphBatch, GradhSphTree
    gbuild.build()
    lib = _native.load()
    boxes = ics_mod.kh_ensemble(64, 4096, 131072, seed=2024 + rank)
    ntot = sum(len(b["x"]) for b in boxes)
    trees = []
    for c in boxes:
        c = dict(c)
        params = c.pop("params")
        t = GradhSphTree(params, precision="mixed", device=local)
        t.set_particles(c)
        trees.append(t)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    batch = GradhSphBatch(trees)
    with ClockSampler(local) as clk:
        for _ in range(args.warmup):
            batch.step()
        ms_batch = 0.0
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            batch.step()
            ms_batch += batch.stats()["ms"]
        # the same simulations one after another, each replayed from its own graph
        for t in trees:
            t.step(graph=True)
        torch.cuda.synchronize()
        ms_seq = 0.0
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        stream = torch.cuda.current_stream()
        for t in trees:
            t.set_stream(stream.cuda_stream)
        for _ in range(args.steps):
            flush.zero_()
            ev0.record(stream)
            for t in trees:
                t.step(graph=True)
            ev1.record(stream)
            torch.cuda.synchronize()
            ms_seq += ev0.elapsed_time(ev1)
    clocks = clk.summary()
    ms_batch = max_over_ranks(ms_batch, world)
    counts = {k: sum(t.stats()[k] for t in trees) for k in ("density_pairs", "hydro_pairs", "exact_checks")}
    flops = counts["density_pairs"] * FLOPS["density"] + counts["hydro_pairs"] * FLOPS["hydro"]
    peak_gf = lib.gsph_fma_peak_gflops(local, 0)
    achieved = flops / (ms_batch / args.steps * 1e-3) / 1e12
    # end to end: host SoA in, batch step, per-box results out
    keys = ("x", "y", "z", "vx", "vy", "vz", "m", "u", "h")
    hbytes = 0
    t0 = time.perf_counter()
    k_e2e = max(1, min(args.steps, 3))
    for _ in range(k_e2e):
        for t, c in zip(trees, boxes):
            t.set_particles({k: c[k] for k in keys})
        batch.step()
        for t in trees:
            for f in ("h", "rho", "ax", "ay", "az", "dudt"):
                t.field(f)
    wall = time.perf_counter() - t0
    hbytes_in = ntot * 8 * len(keys)
    hbytes_out = ntot * 8 * 6
    launches = batch.stats()["launches"]
    batch.close()
    for t in trees:
        t.close()
    value = job_throughput(ntot * args.steps, ms_batch, world)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_batch / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 pairs / f64 positions", "data": "synthetic",
            "config": {"workload": "kh_ensemble", "boxes": 64, "n_total": ntot,
                       "n_per_box": [min(len(b["x"]) for b in boxes), max(len(b["x"]) for b in boxes)],
                       "box": [1.0, 1.0, 0.25], "boundaries": "periodic", "nleafmax": 8, "precision": "mixed",
                       "cuda_graph": True, "l2": "flushed between timed steps (256 MiB write)",
                       "parallelism": f"replicas{world}"},
            "e2e": {"value": world * ntot * k_e2e / wall, "unit": UNIT, "h2d_bytes_per_step": hbytes_in,
                    "d2h_bytes_per_step": hbytes_out,
                    "path": "gsph_set_particles + gsph_batch_step + gsph_get_field per box"},
            "gpu_launches": launches * args.steps,
            "roofline": {"bound": "fp32", "kernel": "whole batch step (density + hydro)", "achieved": achieved,
                         "peak": peak_gf / 1e3, "unit": "TFLOP/s", "frac": achieved / (peak_gf / 1e3),
                         "traffic": None, "peak_source": "measured FMA-loop throughput (gsph_fma_peak_gflops)"},
            "sequential": {"value": world * ntot * args.steps / (ms_seq * 1e-3), "ms_per_step": ms_seq / args.steps,
                           "how": "the 64 simulations stepped one after another, each from its own CUDA graph"},
            "speedup_batch_over_sequential": ms_seq / ms_batch, "counts": counts, "clocks": clocks}
    if rank == 0:
        print(json.dumps(line), flush=True)


def evrard_main(args, rank, world, local):
    """Evrard sphere, N = 8,388,608 gas particles, self-gravity theta = 0.5 quadrupole, plus 64
    stars coupled by FP64 direct sums (gas <- stars, star <- gas tree walk) in every step;
    mixed form with the leaf size chosen by the autotuner, one graph-replayed step per
    timed iteration."""
    import torch
    from gandalf_gb300 import ics as ics_mod
    from gandalf_gb300 import _native
    from gandalf_gb300 import build as gbuild
    from gandalf_gb300.autotune import tune_leaf_size
    from gandalf_gb300.sph import GradhSphTree
    gbuild.build()
    lib = _native.load()
    n = args.n or 8388608
    c = ics_mod.evrard_sphere(n, seed=51 + rank)
    params = c.pop("params")
    form = "mixed" if args.precision == "auto" else args.precision
    steps = args.steps
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    with ClockSampler(local) as clk:
        tune = ({"nleafmax": args.nleafmax} if args.nleafmax > 0 else
                tune_leaf_size(c, params, precision=form, steps=1, device=local))
        t = GradhSphTree(params, precision=form, nleafmax=tune["nleafmax"], device=local)
        if args.nleafmax <= 0:
            t.set_tuning(**{k: tune[k] for k in ("near_depth", "cell_depth", "gather_depth")})
        stream = torch.cuda.current_stream()
        t.set_stream(stream.cuda_stream)
        t.set_particles(c)
        for _ in range(max(1, args.warmup)):
            t.step(graph=True)
        torch.cuda.synchronize()
        ms = 0.0
        for _ in range(steps):
            flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            t.step(graph=True)
            b.record(stream)
            torch.cuda.synchronize()
            ms += a.elapsed_time(b)
        st = t.stats()
        sf = t.star_forces()
    clocks = clk.summary()
    t.close()
    ms = max_over_ranks(ms, world)
    value = job_throughput(n * steps, ms, world)
    flops = (st["density_pairs"] * FLOPS["density"] + st["hydro_pairs"] * FLOPS["hydro_grav"] +
             st["direct_pairs"] * FLOPS["direct"] + st["cell_pairs"] * FLOPS["quad"])
    peak_gf = lib.gsph_fma_peak_gflops(local, 0 if form == "mixed" else 1)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": steps,
            "warmup": args.warmup, "ms_per_step": ms / steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 pairs / f64 positions" if form == "mixed" else "f64",
            "data": "synthetic",
            "config": {"workload": "evrard_sphere", "n": n, "nstar": 64, "star_mass": 1e-3, "star_h": 0.01,
                       "thetamaxsqd": 0.25, "multipole": "quadrupole", "precision": form,
                       ("nleafmax" if args.nleafmax > 0 else "autotuned"): tune, "cuda_graph": True, "parallelism": f"replicas{world}",
                       "l2": "flushed between timed steps (256 MiB write)"},
            "gpu_launches": st["launches"],
            "counts": {k: st[k] for k in ("density_pairs", "hydro_pairs", "direct_pairs", "cell_pairs")},
            "heavy_leaves": {"density": st["heavy_density"], "forces": st["heavy_forces"]},
            "phases_ms_last_step": {k: st[k] for k in ("ms_build", "ms_density", "ms_hmax", "ms_forces")},
            "star_gpot_mean": float(np.mean(sf["gpot"])),
            "roofline": {"bound": "fp32" if form == "mixed" else "fp64", "kernel": "whole step",
                         "achieved": flops / (ms / steps * 1e-3) / 1e12, "peak": peak_gf / 1e3, "unit": "TFLOP/s",
                         "frac": flops / (ms / steps * 1e-3) / 1e12 / (peak_gf / 1e3), "traffic": None,
                         "peak_source": "measured FMA-loop throughput (gsph_fma_peak_gflops)"},
            "clocks": clocks}
    if rank == 0:
        print(json.dumps(line), flush=True)


def kdk_workload(n, rank=0):
    from gandalf_gb300 import ics as ics_mod
    c = ics_mod.rotating_cloud(n, seed=31 + rank)
    params = c.pop("params")
    kdk = c.pop("kdk")
    return c, params, kdk


def kdk_config(n, kdk, K):
    """The workload keys of the rotating-cloud line (shared by both arms)."""
    return {"workload": "rotating_cloud", "n": n, "nlevels": kdk["nlevels"], "kdk_steps": K,
            "level_diff_max": kdk["level_diff_max"], "courant_mult": kdk["courant_mult"],
            "accel_mult": kdk["accel_mult"], "eos": "isothermal", "thetamaxsqd": 0.25, "multipole": "quadrupole",
            "gravity_mac": "geometric", "nleafmax": 8, "h_fac": 1.2, "h_converge": 0.01, "kernel": "m4",
            "unit_of_work": "active particle through one h solve and force pass (per KDK substep)"}


def err_stats(a, b, floor_frac=1e-6):
    """(RMS, max) of |a - b| / (|b| + floor_frac rms b) over all particles."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    floor = floor_frac * np.sqrt(np.mean(b * b)) + 1e-300
    e = np.abs(a - b) / (np.abs(b) + floor)
    return {"rms": float(np.sqrt(np.mean(e * e))), "max": float(e.max())}


def vec_err_stats(a, b, keys):
    A = np.stack([a[k] for k in keys], 1)
    B = np.stack([b[k] for k in keys], 1)
    nb = np.linalg.norm(B, axis=1)
    floor = 1e-6 * np.sqrt(np.mean(nb * nb)) + 1e-300
    e = np.linalg.norm(A - B, axis=1) / (nb + floor)
    return {"rms": float(np.sqrt(np.mean(e * e))), "max": float(e.max())}


def all_errors(a, b):
    """Mixed against FP64 for every per-particle result.  div v and du/dt can be zero up to
    rounding noise (solid-body rotation), so their errors are taken against their natural
    scales, the sound-crossing rate c_s / h and u c_s / h (RMS over particles)."""
    out = {k: err_stats(a[k], b[k]) for k in ("h", "rho", "invomega", "zeta", "pressure", "sound", "gpot")
           if k in a}
    rate = b["sound"] / b["h"]
    for k, scale in (("div_v", rate), ("dudt", b["u"] * rate)):
        if k in a:
            d = np.abs(np.asarray(a[k]) - np.asarray(b[k])) / np.sqrt(np.mean(scale * scale))
            out[k] = {"rms": float(np.sqrt(np.mean(d * d))), "max": float(d.max()),
                      "normalised_by": "rms of c_s/h" if k == "div_v" else "rms of u c_s/h"}
    out["a"] = vec_err_stats(a, b, ("ax", "ay", "az"))
    out["a_tree"] = vec_err_stats(a, b, ("agx", "agy", "agz"))
    return out


def csr_differ(oa, ia, ob, ib):
    """Particles whose neighbour sets (CSR, any order inside a row) differ."""
    n = len(oa) - 1
    ca, cb = np.diff(oa), np.diff(ob)
    differ = ca != cb
    same = ~differ
    rows_a = np.repeat(np.arange(n), ca)
    rows_b = np.repeat(np.arange(n), cb)
    sa = ia[np.lexsort((ia, rows_a))]
    sb = ib[np.lexsort((ib, rows_b))]
    keep_a = same[rows_a]
    keep_b = same[rows_b]
    bad = sa[keep_a] != sb[keep_b]
    if bad.any():
        differ[np.unique(rows_a[keep_a][bad])] = True
    return int(differ.sum())


def precision_step(c, params, h_converge=None, record=True):
    """One full step (tree, h solve, forces) of both forms from identical inputs: errors of
    every quantity, and how many particles' interaction lists differ between the forms."""
    from gandalf_gb300.sph import GradhSphTree
    prm = dict(params)
    if h_converge is not None:
        prm["h_converge"] = h_converge
    res, lists = {}, {}
    for form in ("fp64", "mixed", "mixed_compensated"):
        kw = {"precision": "mixed", "compensated": 1} if form == "mixed_compensated" else {"precision": form}
        t = GradhSphTree(prm, device=int(os.environ.get("LOCAL_RANK", "0")), **kw)
        if record:
            t.set_recording(True, 512)
        t.set_particles(c)
        t.step()
        res[form] = t.results()
        if record and form != "mixed_compensated":
            lists[form] = (t.sph_neighbours_csr(), t.direct_summary(), t.cell_summary())
        res[form]["exact_checks"] = t.stats()["exact_checks"]
        t.close()
    out = {"errors": all_errors(res["mixed"], res["fp64"]),
           "errors_compensated": all_errors(res["mixed_compensated"], res["fp64"]),
           "exact_checks_mixed": int(res["mixed"]["exact_checks"])}
    if record:
        (oa, ia), (dca, dha), (_, cca, cha) = lists["mixed"]
        (ob, ib), (dcb, dhb), (_, ccb, chb) = lists["fp64"]
        out["list_diff"] = {"sph_particles": csr_differ(oa, ia, ob, ib),
                            "direct_particles": int(np.sum((dca != dcb) | (dha != dhb))),
                            "multipole_leaves": int(np.sum((cca != ccb) | (cha != chb))),
                            "n": len(oa) - 1}
    return out


def run_kdk_form(c, params, kdk, form, K, warm_seq, stream, device, graph=True):
    """Warm-up sequences (setup + K graph-replayed steps), then the timed one: setup
    outside, the K steps between CUDA events on the stream.  Returns the context open."""
    import torch
    from gandalf_gb300.sph import GradhSphTree
    if form == "mixed_compensated":
        t = GradhSphTree(params, precision="mixed", compensated=1, device=device)
    else:
        t = GradhSphTree(params, precision=form, device=device)
    t.set_stream(stream.cuda_stream)
    for _ in range(warm_seq):
        t.set_particles(c)
        t.kdk_setup(**kdk)
        t.kdk_steps(K, graph=graph)         # the first call captures the K-step graph
    t.set_particles(c)
    t.kdk_setup(**kdk)
    torch.cuda.synchronize()
    u0 = t.kdk_status()["active_updates"]
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    t.kdk_steps(K, graph=graph)
    ev1.record(stream)
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1)
    st = t.kdk_status()
    s2 = t.stats()
    tm = t.kdk_timing()
    upd = st["active_updates"] - u0
    n = len(c["x"])
    return t, {"value": upd / (ms * 1e-3), "ms_total": ms, "ms_per_step": ms / K, "active_updates": upd,
               "active_fraction_per_step": upd / (K * n), "level_max": st["level_max"], "t_end": st["t"],
               "phases_ms_first_passes": {"build": tm["ms_build"], "density": tm["ms_density"],
                                          "forces": tm["ms_forces"]},
               "repeat_passes_run": tm["repeat_passes"],
               "counts": {k: s2[k] for k in ("density_pairs", "hydro_pairs", "direct_pairs", "cell_pairs",
                                             "exact_checks", "heavy_density", "heavy_forces")},
               "counts_first_passes": {k: tm[k] for k in ("density_pairs", "hydro_pairs", "direct_pairs",
                                                           "cell_pairs")},
               "launches": s2["launches"]}


def kdk_e2e(t, c, kdk, K):
    """Through the C ABI on an open context: pinned host arrays in, setup, K steps (the
    captured graph), positions, velocities and solved fields out into pinned arrays."""
    import torch
    keys = ("x", "y", "z", "vx", "vy", "vz", "m", "u", "h")
    pin = {k: torch.from_numpy(np.ascontiguousarray(c[k], dtype=np.float64)).pin_memory().numpy() for k in keys}
    outs = ("x", "y", "z", "vx", "vy", "vz")
    fields = ("h", "rho", "u", "ax", "ay", "az", "gpot")
    n = len(c["x"])
    obuf = {k: torch.empty(n, dtype=torch.float64).pin_memory().numpy() for k in outs + fields}
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    t.set_particles(pin)
    t.kdk_setup(**kdk)
    u0 = t.kdk_status()["active_updates"]
    t.kdk_steps(K, graph=True)
    for k in outs:
        t.kdk_state(k, out=obuf[k])
    for k in fields:
        t.field(k, out=obuf[k])
    wall = time.perf_counter() - t0
    upd = t.kdk_status()["active_updates"] - u0
    return {"value": upd / wall, "wall_s": wall, "h2d_bytes_per_step": n * 8 * len(keys) / K,
            "d2h_bytes_per_step": n * 8 * (len(outs) + len(fields)) / K,
            "path": "gsph_set_particles (pinned host arrays) + gsph_kdk_setup + gsph_kdk_steps(K, graph) + "
                    "gsph_kdk_get_state / gsph_get_field into pinned arrays; the setup (two h solves and a "
                    "force pass) is inside the timed span, its updates are not counted"}


def kdk_cpu_baseline(c, params, kdk, nsteps=2):
    from oracle import oracle
    cores = os.cpu_count() or 1
    r = oracle.kdk(c, params, kdk, nsteps, nthreads=cores)
    return {"value": r["step_updates"] / r["steps_s"], "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"setup + {nsteps} KDK main-loop steps of the same {len(c['x'])}-particle cloud "
                      f"(oracle/gsph_oracle.cpp, the C++/OpenMP restatement of the reference path); the "
                      f"{nsteps} steps timed: {r['step_updates']} active updates in {r['steps_s']:.2f} s"}


def kdk_main(args, rank, world, local):
    """Rotating isothermal cloud, N = 1,048,576, self-gravity theta = 0.5 quadrupole, 4
    block-timestep levels: K KDK main-loop steps replayed from one CUDA graph, FP64 and
    mixed forms.  The unit of work is one active particle through one h solve and force
    pass (the metric's unit for block-timestep configurations)."""
    import torch
    from gandalf_gb300 import _native
    from gandalf_gb300 import build as gbuild
    gbuild.build()
    lib = _native.load()
    n = args.n or 1048576
    K = args.steps or 20
    W = args.warmup
    c, params, kdk = kdk_workload(n, rank)
    stream = torch.cuda.current_stream()
    forms = ["fp64", "mixed", "mixed_compensated"] if args.precision == "auto" else [args.precision]
    warm_seq = max(1, -(-W // K))           # whole K-step sequences covering >= W warm-up steps
    out, finals = {}, {}
    ctx_head = None
    head = "mixed" if "mixed" in forms else forms[0]
    with ClockSampler(local) as clk:
        for form in forms:
            if world > 1:
                import torch.distributed as dist
                dist.barrier()
            t, R = run_kdk_form(c, params, kdk, form, K, warm_seq, stream, local, graph=not args.no_graph)
            finals[form] = t.results()
            for k in ("x", "y", "z"):
                finals[form]["pos_" + k] = t.kdk_state(k)
            out[form] = R
            if form == head:
                ctx_head = t
            else:
                t.close()
    clocks = clk.summary()
    R = out[head]
    ms_job = max_over_ranks(R["ms_total"], world)
    value = job_throughput(R["active_updates"], ms_job, world)
    cnt = R["counts_first_passes"]
    fp64 = head == "fp64"
    peak_gf = lib.gsph_fma_peak_gflops(local, 1 if fp64 else 0)
    f_force = (cnt["hydro_pairs"] * FLOPS["hydro_grav"] + cnt["direct_pairs"] * FLOPS["direct"] +
               cnt["cell_pairs"] * FLOPS["quad"])
    f_dens = cnt["density_pairs"] * FLOPS["density"]
    passes = K                        # the first force pass of every step, event-timed
    ms_f = R["phases_ms_first_passes"]["forces"]
    ms_d = R["phases_ms_first_passes"]["density"]
    traffic = FORCE_TRAFFIC.get(("rotating_cloud", n, head))
    roof = {"bound": "fp64" if fp64 else "fp32",
            "kernel": "force pass (k_all_forces_mixed + heavy-leaf k_all_forces_mixed_wide)" if not fp64
            else "force pass (k_all_forces_fp64)",
            "achieved": f_force / (ms_f * 1e-3) / 1e12, "peak": peak_gf / 1e3, "unit": "TFLOP/s",
            "frac": (f_force / (ms_f * 1e-3) / 1e12) / (peak_gf / 1e3),
            "traffic": traffic["bytes"] if traffic else None,
            "traffic_source": traffic["source"] if traffic else None,
            "peak_source": "FMA-loop throughput measured live on this GPU (gsph_fma_peak_gflops); "
                           "the pair loops run on the FP32/FP64 pipes, not HBM or tensor cores",
            "flops_per_launch": f_force / passes, "ms_per_launch": ms_f / passes, "launches": passes,
            "timing": "CUDA events recorded inside the K-step graph around the first force pass of every "
                      "step, summed; flops from the interaction counts of those passes (the CheckTimesteps "
                      "repeat passes are conditional graph nodes, which hold no events)"}
    roof_d = {"bound": roof["bound"], "kernel": "h solve (k_density_mixed + heavy-leaf k_density_mixed_pp, "
              "with the hmax update and mirror refresh)" if not fp64 else "h solve (k_density_fp64)",
              "achieved": f_dens / (ms_d * 1e-3) / 1e12, "peak": peak_gf / 1e3, "unit": "TFLOP/s",
              "frac": (f_dens / (ms_d * 1e-3) / 1e12) / (peak_gf / 1e3), "ms_total": ms_d}
    cfg = kdk_config(n, kdk, K)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K, "warmup": W,
            "ms_per_step": ms_job / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if fp64 else "f32 pairs / f64 positions, h iteration and moments",
            "data": "synthetic (seeded rotating-cloud generator, no dataset)", "config": cfg,
            "run": {"precision": head, "cuda_graph": "stream launches" if args.no_graph else "K steps in one graph",
                    "warmup_sequences": warm_seq, "warmup_kdk_steps": warm_seq * K,
                    "l2": "working set (1M particles, ~0.6 GB) larger than L2; not flushed",
                    "parallelism": f"replicas{world}"},
            "gpu_launches": R["launches"], "roofline": roof, "roofline_density": roof_d,
            "forms": out, "clocks": clocks}
    if "fp64" in out and "mixed" in out:
        line["speedup_mixed_over_fp64"] = out["mixed"]["value"] / out["fp64"]["value"]
        a, b = finals["mixed"], finals["fp64"]
        errs = all_errors(a, b)
        pos = np.sqrt(np.mean(sum((a["pos_" + k] - b["pos_" + k]) ** 2 for k in ("x", "y", "z"))))
        errs["position_rms_abs"] = float(pos)
        line["mixed_vs_fp64_after_all_steps"] = errs
    if "fp64" in out and "mixed_compensated" in out:
        a, b = finals["mixed_compensated"], finals["fp64"]
        line["mixed_compensated_vs_fp64_after_all_steps"] = all_errors(a, b)
        line["compensated_cost"] = out["mixed_compensated"]["ms_total"] / out["mixed"]["ms_total"] - 1.0
    if not args.no_e2e and ctx_head is not None:
        e = kdk_e2e(ctx_head, c, kdk, K)
        line["e2e"] = {"value": world * e["value"], "unit": UNIT, "h2d_bytes_per_step": e["h2d_bytes_per_step"],
                       "d2h_bytes_per_step": e["d2h_bytes_per_step"], "path": e["path"], "wall_s": e["wall_s"]}
    if ctx_head is not None:
        ctx_head.close()
    if rank == 0 and not args.no_precision and "fp64" in out and "mixed" in out:
        # identical inputs, one full step: every quantity and the lists, at the reference's
        # default h_converge and at 1e-10 (which leaves no room for iteration-path flips)
        line["precision_one_step"] = {"h_converge_0.01": precision_step(c, params),
                                      "h_converge_1e-10": precision_step(c, params, 1e-10, record=False)}
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = kdk_cpu_baseline(c, params, kdk)
    if rank == 0:
        print(json.dumps(line), flush=True)


def workload(name, n):
    from gandalf_gb300 import ics
    if name == "plummer_sphere":
        return ics.plummer_sphere(n or 262144, seed=4321)
    if name == "periodic_cube":
        return ics.periodic_cube(n or 32768, seed=1234)
    raise SystemExit(f"unknown workload {name}")


def workload_config(name, c):
    p = c["params"]
    cfg = {"workload": name, "n": len(c["x"]), "nleafmax": 8, "h_fac": 1.2, "h_converge": 0.01,
           "kernel": "m4", "alpha_visc": 1.0, "beta_visc": 2.0}
    if p.get("self_gravity"):
        cfg.update(thetamaxsqd=p["thetamaxsqd"], multipole="quadrupole", gravity_mac="geometric")
    else:
        cfg.update(boundaries="periodic")
    return cfg


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms while running."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = max(smax, float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def gradh_record_dtype():
    """GradhSphParticle<3>'s field order and sizes (src/Headers/Particle.h:133-368)."""
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


def gradh_records(c):
    """Page-locked host records laid out like GradhSphParticle<3>."""
    import torch
    dt = gradh_record_dtype()
    n = len(c["x"])
    buf = torch.empty(n * dt.itemsize, dtype=torch.uint8, pin_memory=True)
    rec = buf.numpy().view(dt)
    rec[:] = np.zeros(1, dtype=dt)
    rec["r"] = np.stack([c["x"], c["y"], c["z"]], 1)
    rec["v"] = np.stack([c["vx"], c["vy"], c["vz"]], 1)
    rec["m"], rec["u"], rec["h"] = c["m"], c["u"], c["h"]
    rec["iorig"] = np.arange(n)
    rec["alpha"] = 1.0
    off = {k: dt.fields[k][1] for k in ("r", "v", "m", "h", "u", "rho", "invomega", "zeta", "hfactor",
                                         "hrangesqd", "pressure", "sound", "div_v", "dudt", "a",
                                         "atree", "gpot", "gpot_hydro")}
    return buf, rec, off


def algorithmic_flops(st, gravity, quad=True):
    """(flops of the force kernel, flops of the density kernel) from the interaction counts."""
    if gravity:
        fk = (st["hydro_pairs"] * FLOPS["hydro_grav"] + st["direct_pairs"] * FLOPS["direct"] +
              st["cell_pairs"] * (FLOPS["quad"] if quad else FLOPS["mono"]))
    else:
        fk = st["hydro_pairs"] * FLOPS["hydro"]
    return fk, st["density_pairs"] * FLOPS["density"]


def run_form(c, params, precision, steps, warmup, flush, graph=True):
    import torch
    from gandalf_gb300.sph import GradhSphTree

    dev = {k: torch.from_numpy(np.ascontiguousarray(c[k])).cuda() for k in
           ("x", "y", "z", "vx", "vy", "vz", "m", "u", "h")}
    t = GradhSphTree(params, precision=precision, device=torch.cuda.current_device())
    stream = torch.cuda.current_stream()
    t.set_stream(stream.cuda_stream)
    for _ in range(warmup):
        t.set_particles(dev)
        t.step(graph=graph)
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    per = {"ms_build": 0.0, "ms_density": 0.0, "ms_hmax": 0.0, "ms_forces": 0.0}
    launches = 0
    st = None
    for k in range(steps):
        flush.zero_()                      # L2 flush, outside the timed pair
        ev[k][0].record(stream)
        t.set_particles(dev)
        t.step(graph=graph)
        ev[k][1].record(stream)
        st = t.stats()
        for key in per:
            per[key] += st[key]
        launches += st["launches"]
    torch.cuda.synchronize()
    ms = sum(a.elapsed_time(b) for a, b in ev)
    out = t.results()
    t.close()
    return {"ms_total": ms, "per": {k: v / steps for k, v in per.items()}, "stats": st,
            "launches": launches, "results": out}


def run_e2e(c, params, precision, steps, warmup, graph=True):
    """Records in, step, records out through the C ABI; separate pinned input and output
    record buffers so every step starts from the same inputs, as the device-resident
    loop does."""
    from gandalf_gb300.sph import GradhSphTree
    import torch
    buf, rec, off = gradh_records(c)
    obuf, orec, _ = gradh_records(c)
    t = GradhSphTree(params, precision=precision, device=torch.cuda.current_device())
    for _ in range(max(1, warmup)):
        t.set_particles_aos(rec, off)
        t.step(graph=graph)
        t.get_particles_aos(orec, off)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        t.set_particles_aos(rec, off)
        t.step(graph=graph)
        t.get_particles_aos(orec, off)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    t.close()
    n = len(rec)
    # in: the whole records are copied; out: page-locked records are written in place by a
    # kernel, the 19 output doubles of each particle (h, u, rho, invomega, zeta, hfactor,
    # hrangesqd, pressure, sound, div_v, dudt, gpot, gpot_hydro, a, atree)
    return {"wall": wall, "bytes": n * rec.dtype.itemsize, "bytes_out": n * 19 * 8}


def cpu_baseline(c, params, budget_s=40.0):
    from oracle import oracle
    cores = os.cpu_count() or 1
    t0 = time.perf_counter()
    oracle.run(c, params, nthreads=cores)
    wall = time.perf_counter() - t0
    return {"value": len(c["x"]) / wall, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"one full step of the {len(c['x'])}-particle workload "
                      f"(tree build + h solve + forces), {wall:.2f} s wall"}


def kdk_reference_arm(args):
    """The same K main-loop steps, after the same setup, by the CPU restatement of the
    reference on all host threads; the K steps are timed."""
    from oracle import oracle
    n = args.n or 1048576
    K = args.steps or 20
    c, params, kdk = kdk_workload(n, 0)
    cores = os.cpu_count() or 1
    r = oracle.kdk(c, params, kdk, K, nthreads=cores)
    value = r["step_updates"] / r["steps_s"]
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": K,
            "warmup": args.warmup, "ms_per_step": 1e3 * r["steps_s"] / K, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded rotating-cloud generator, no dataset)", "config": kdk_config(n, kdk, K),
            "impl": "reference", "status": r["status"],
            "active_fraction_per_step": r["step_updates"] / (K * n),
            "setup_s": r["setup_s"],
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"setup (untimed warm-up) + {K} KDK main-loop steps of the {n}-particle "
                                       f"cloud on {cores} host threads (oracle/gsph_oracle.cpp, the C++/OpenMP "
                                       f"restatement of the reference path); {r['step_updates']} active updates "
                                       f"in {r['steps_s']:.1f} s"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def reference_arm(args):
    from oracle import oracle
    if args.workload == "rotating_cloud":
        return kdk_reference_arm(args)
    c = workload(args.workload, args.n)
    params = dict(c["params"])
    cores = os.cpu_count() or 1
    n = len(c["x"])
    t0 = time.perf_counter()
    oracle.run(c, params, nthreads=cores)          # first warm-up step sizes the run
    t_one = time.perf_counter() - t0
    budget = 150.0
    warm = min(max(args.warmup - 1, 0), int(budget / 3 / max(t_one, 1e-3)))
    for _ in range(warm):
        oracle.run(c, params, nthreads=cores)
    k = max(1, min(args.steps, int(budget / max(t_one, 1e-3))))
    t0 = time.perf_counter()
    for _ in range(k):
        oracle.run(c, params, nthreads=cores)
    wall = time.perf_counter() - t0
    value = n * k / wall
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * wall / k, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(args.workload, c), "impl": "reference",
            "steps_executed": k,
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"{k} full steps of the {n}-particle workload on {cores} host threads "
                                       "(oracle/gsph_oracle.cpp, the C++ restatement of the reference path)"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        if rank == 0:
            reference_arm(args)
        return
    import torch
    import torch.distributed as dist
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    if args.workload == "evrard_sphere":
        evrard_main(args, rank, world, local)
        if world > 1:
            dist.destroy_process_group()
        return
    if args.workload == "rotating_cloud":
        kdk_main(args, rank, world, local)
        if world > 1:
            dist.destroy_process_group()
        return
    if args.workload == "kh_ensemble":
        ensemble_main(args, rank, world, local)
        if world > 1:
            dist.destroy_process_group()
        return
    from gandalf_gb300 import _native
    from gandalf_gb300 import build as gbuild
    gbuild.build()
    lib = _native.load()
    c = workload(args.workload, args.n)
    params = dict(c["params"])
    gravity = bool(params.get("self_gravity"))
    n = len(c["x"])
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    forms = ["fp64", "mixed"] if args.precision == "auto" else [args.precision]
    results = {}
    with ClockSampler(local) as clk:
        for form in forms:
            try:
                if world > 1:
                    dist.barrier()
                torch.cuda.synchronize()
                results[form] = run_form(c, params, form, args.steps, args.warmup, flush, not args.no_graph)
                if world > 1:
                    dist.barrier()
                torch.cuda.synchronize()
            except RuntimeError as e:
                if args.precision != "auto":
                    raise
                results[form] = {"error": str(e)}
    clocks = clk.summary()
    ok = [f for f in forms if "error" not in results[f]]
    head = "mixed" if "mixed" in ok else ok[0]
    R = results[head]
    ms = max_over_ranks(R["ms_total"], world)
    value = job_throughput(n * args.steps, ms, world)
    e2e = None
    if not args.no_e2e:
        E = run_e2e(c, params, head, max(1, min(args.steps, 5)), 1, not args.no_graph)
        k = max(1, min(args.steps, 5))
        e2e = {"value": n * k / E["wall"] * world, "unit": UNIT, "h2d_bytes_per_step": E["bytes"],
               "d2h_bytes_per_step": E["bytes_out"], "path": "gsph_set_particles_aos + gsph_step + "
               "gsph_get_particles_aos, pinned host records (records copied in whole; the output fields "
               "written in place)"}
    st = R["stats"]
    f_force, f_dens = algorithmic_flops(st, gravity)
    fp64 = head == "fp64"
    peak_gf = lib.gsph_fma_peak_gflops(local, 1 if fp64 else 0)
    achieved = f_force / (R["per"]["ms_forces"] * 1e-3) / 1e12
    roof = {"bound": "fp64" if fp64 else "fp32", "kernel": "all-forces" if gravity else "hydro-forces",
            "achieved": achieved, "peak": peak_gf / 1e3, "unit": "TFLOP/s",
            "frac": achieved / (peak_gf / 1e3) if peak_gf > 0 else None,
            "traffic": (FORCE_TRAFFIC.get((args.workload, n, head)) or {}).get("bytes"),
            "traffic_source": (FORCE_TRAFFIC.get((args.workload, n, head)) or {}).get("source"),
            "peak_source": "measured FMA-loop throughput of this GPU (gsph_fma_peak_gflops); "
                           "MEASURED_PEAKS.json holds HBM and bf16 figures only",
            "flops_per_launch": f_force, "ms_per_launch": R["per"]["ms_forces"]}
    forms_out = {}
    for f in forms:
        if "error" in results[f]:
            forms_out[f] = {"error": results[f]["error"][:200]}
            continue
        Rf = results[f]
        forms_out[f] = {"value": n * args.steps / (Rf["ms_total"] * 1e-3),
                        "ms_per_step": Rf["ms_total"] / args.steps,
                        "phases_ms": {k: round(v, 4) for k, v in Rf["per"].items()},
                        "counts": {k: Rf["stats"][k] for k in ("density_pairs", "hydro_pairs",
                                                               "direct_pairs", "cell_pairs",
                                                               "exact_checks", "launches")},
                        "heavy_leaves": {"density": Rf["stats"]["heavy_density"],
                                         "forces": Rf["stats"]["heavy_forces"]}}
    if "fp64" in ok and "mixed" in ok:
        forms_out["mixed_vs_fp64_rel_err"] = all_errors(results["mixed"]["results"], results["fp64"]["results"])
        forms_out["speedup_mixed_over_fp64"] = results["fp64"]["ms_total"] / results["mixed"]["ms_total"]
    cfg = workload_config(args.workload, c)
    run = {"precision": head, "cuda_graph": not args.no_graph,
           "l2": "flushed between timed steps (256 MiB write, outside the timed span)",
           "parallelism": f"replicas{world}"}
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64" if fp64 else "f32 pairs / f64 positions",
            "data": "synthetic", "config": cfg, "run": run, "e2e": e2e, "gpu_launches": R["launches"],
            "roofline": roof, "forms": forms_out, "clocks": clocks}
    if rank == 0 and not args.no_precision and "fp64" in ok and "mixed" in ok:
        line["precision_one_step"] = {"h_converge_0.01": precision_step(c, params),
                                      "h_converge_1e-10": precision_step(c, params, 1e-10, record=False)}
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(c, params)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
