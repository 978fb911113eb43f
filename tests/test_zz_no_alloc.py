"""The allocation-free KD-tree ordering entry point against the regular build.

gsph_kdtree_order_noalloc serves callers that may not allocate device memory (their
device memory belongs to their own pool allocator, or they run a time-critical loop
that cannot absorb cudaMalloc's device synchronisation).  It must give exactly the leaf
order gsph_build_tree gives — an integer permutation, so the comparison is exact — on
two calls in a row sharing its fixed scratch array, and refuse sizes beyond its limit.
This file is collected last so that a failure here comes after every other test.
"""
import ctypes

import numpy as np
import pytest

from gandalf_gb300 import _native
from gandalf_gb300 import ics as ics_mod
from gandalf_gb300.sph import GradhSphTree

pytestmark = pytest.mark.gpu

MAX_N = 32768


def regular_order(c, nleafmax=8):
    t = GradhSphTree(c["params"], nleafmax=nleafmax)
    t.set_particles(c)
    t.BuildTree()
    order = t.tree()["order"]
    t.close()
    return order


def noalloc_order(lib, c, nleafmax=8):
    import torch
    dev = {k: torch.from_numpy(np.ascontiguousarray(c[k])).cuda() for k in ("x", "y", "z", "h")}
    out = torch.full((len(c["x"]),), -1, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()
    rc = lib.gsph_kdtree_order_noalloc(ctypes.c_void_p(dev["x"].data_ptr()), ctypes.c_void_p(dev["y"].data_ptr()),
                                       ctypes.c_void_p(dev["z"].data_ptr()), ctypes.c_void_p(dev["h"].data_ptr()),
                                       len(c["x"]), nleafmax, ctypes.c_void_p(out.data_ptr()),
                                       ctypes.c_void_p(stream.cuda_stream))
    torch.cuda.synchronize()
    return rc, out.cpu().numpy()


def test_noalloc_order_matches_regular_build_twice():
    import torch
    torch.cuda.init()
    lib = _native.load()
    cases = [ics_mod.plummer_sphere(MAX_N, seed=31), ics_mod.periodic_cube(5000, seed=32)]
    for c in cases:
        want = regular_order(c)
        for _ in range(2):                      # two calls in a row share the scratch
            rc, got = noalloc_order(lib, c)
            assert rc == 0
            assert np.array_equal(got, want)


def test_noalloc_order_at_the_depth_limit():
    """Nleafmax 1 and 8,192 particles: a 13-level tree, the deepest the fixed scratch
    holds (heap indices up to 16,382, 4,096 segments on the last level)."""
    import torch
    torch.cuda.init()
    lib = _native.load()
    c = ics_mod.plummer_sphere(8192, seed=35)
    want = regular_order(c, nleafmax=1)
    for _ in range(2):
        rc, got = noalloc_order(lib, c, nleafmax=1)
        assert rc == 0
        assert np.array_equal(got, want)


def test_noalloc_rejects_sizes_beyond_its_limit():
    import torch
    torch.cuda.init()
    lib = _native.load()
    c = ics_mod.plummer_sphere(MAX_N + 1, seed=33)
    rc, got = noalloc_order(lib, c)
    assert rc == -6                             # GSPH_ERR_CAPACITY
    assert np.all(got == -1)                    # nothing was written
    c = ics_mod.plummer_sphere(8193, seed=36)     # within the particle limit, but 14 levels
    rc, got = noalloc_order(lib, c, nleafmax=1)
    assert rc == -6
    assert np.all(got == -1)
    c = ics_mod.plummer_sphere(1000, seed=34)
    rc, _ = noalloc_order(lib, c, nleafmax=0)
    assert rc == -1                             # GSPH_ERR_INVALID
