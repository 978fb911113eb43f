"""Leaf-size autotuner for a particle set on the GPU.

Nleafmax is the reference's own tree parameter (src/Common/Parameters.cpp:306): it sets how
many particles share one leaf cell, hence one warp of the pair kernels, the length of the
gather and interaction lists and the depth of the tree.  The fastest value depends on the
particle distribution and N, so the tuner times the step (tree build, h solve, forces,
replayed from its CUDA graph) for each candidate on the caller's own particles and keeps
the fastest.  Every candidate is a valid configuration of the reference; results differ
between candidates only as the reference's own results differ with Nleafmax.
"""
from __future__ import annotations

import json
import os

from .sph import GradhSphTree

CANDIDATES = (4, 6, 8, 12, 16)


def tune_leaf_size(ics: dict, params: dict, precision: str = "mixed", candidates=CANDIDATES, steps: int = 2,
                   device: int = 0, cache: str | None = None) -> dict:
    """Time `steps` graph-replayed steps per candidate Nleafmax; returns
    {"nleafmax": best, "ms_per_step": {candidate: ms}}.  With `cache` (a JSON file path), a
    result for the same (N, precision, gravity, periodic) is reused."""
    key = f"{len(ics['x'])}:{precision}:{int(params.get('self_gravity', 0))}:{int(params.get('periodic', 0))}"
    if cache and os.path.exists(cache):
        with open(cache) as f:
            known = json.load(f)
        if key in known:
            return known[key]
    import torch
    timings = {}
    for nl in candidates:
        t = GradhSphTree(params, precision=precision, nleafmax=int(nl), device=device)
        stream = torch.cuda.current_stream()
        t.set_stream(stream.cuda_stream)
        t.set_particles(ics)
        t.step(graph=True)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(steps):
            t.step(graph=True)
        b.record(stream)
        torch.cuda.synchronize()
        timings[int(nl)] = a.elapsed_time(b) / steps
        t.close()
    best = min(timings, key=timings.get)
    res = {"nleafmax": best, "ms_per_step": timings}
    if cache:
        known = {}
        if os.path.exists(cache):
            with open(cache) as f:
                known = json.load(f)
        known[key] = res
        with open(cache, "w") as f:
            json.dump(known, f)
    return res
