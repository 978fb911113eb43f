"""Autotuning of the pair kernels' mapping for a particle set on the GPU.

The search itself is native (gsph_autotune in the C ABI, usable from any host language):
it times the step (tree build, h solve, forces, replayed from its CUDA graph) on the
caller's own particles for candidate leaf sizes (Nleafmax, the reference's own tree
parameter, src/Common/Parameters.cpp:306), near-list depths (how many warps work on one
leaf cell: a deeper near list than the warp holds sends the leaf to the 8-warp kernel),
multipole-list tile depths and density gather-list depths, and keeps the fastest.  Every
candidate is a valid configuration of the reference; results differ between leaf sizes
only as the reference's own results differ with Nleafmax.  This module adds a JSON cache
keyed by the particle set's shape.
"""
from __future__ import annotations

import json
import os

from .sph import GradhSphTree


def tune(ics: dict, params: dict, precision: str = "mixed", steps: int = 2, device: int = 0,
         cache: str | None = None) -> dict:
    """{"nleafmax", "near_depth", "cell_depth", "gather_depth", "tried": [...]} for these
    particles.  With `cache` (a JSON file path), a result for the same (N, precision,
    gravity, periodic) is reused."""
    key = f"{len(ics['x'])}:{precision}:{int(params.get('self_gravity', 0))}:{int(params.get('periodic', 0))}"
    if cache and os.path.exists(cache):
        with open(cache) as f:
            known = json.load(f)
        if key in known:
            return known[key]
    t = GradhSphTree(params, precision=precision, device=device)
    try:
        t.set_particles(ics)
        res = t.autotune(steps)
    finally:
        t.close()
    if cache:
        known = {}
        if os.path.exists(cache):
            with open(cache) as f:
                known = json.load(f)
        known[key] = res
        with open(cache, "w") as f:
            json.dump(known, f)
    return res


def tune_leaf_size(ics: dict, params: dict, precision: str = "mixed", steps: int = 2, device: int = 0,
                   cache: str | None = None) -> dict:
    """The full tuning (see `tune`); kept under its earlier name."""
    return tune(ics, params, precision=precision, steps=steps, device=device, cache=cache)
