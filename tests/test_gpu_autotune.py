"""The native autotuner (gsph_autotune): leaf size, near-list depth (how many warps work on
a leaf cell) and list tile depths, chosen by timing the caller's particles; the tuned
configuration gives the reference's results for its leaf size."""
import numpy as np
import pytest

from gandalf_gb300 import ics as ics_mod
from gandalf_gb300.sph import GandalfError, GradhSphTree
from oracle import oracle
from parity import check_mixed

pytestmark = pytest.mark.gpu


def test_autotune_searches_all_three_dimensions_and_keeps_parity():
    c = ics_mod.plummer_sphere(65536, seed=777)
    params = c["params"]
    t = GradhSphTree(params, precision="mixed")
    t.set_particles(c)
    res = t.autotune(steps=1)
    tried = res["tried"]
    assert {x["nleafmax"] for x in tried} >= {4, 6, 8, 12, 16}
    assert {x["near_depth"] for x in tried} >= {64, 128, 256}
    assert {x["cell_depth"] for x in tried} >= {128, 256, 512}
    assert {x["gather_depth"] for x in tried} >= {64, 128, 256}
    assert all(x["ms_per_step"] > 0 for x in tried)
    best = min(tried, key=lambda x: x["ms_per_step"])
    assert res["nleafmax"] == best["nleafmax"] and t.tuning()["nleafmax"] == res["nleafmax"]
    # the tuned context steps to the reference's results for its leaf size
    t.step()
    got = t.results()
    t.close()
    ref = oracle.run(c, dict(params, nleafmax=res["nleafmax"]))["particles"]
    print(res["nleafmax"], check_mixed(got, ref))


def test_depths_change_speed_not_results():
    """Shallow depths send more leaves to the 8-warp and per-particle kernels; the results
    stay within the mixed form's tolerance of the fp64 oracle."""
    c = ics_mod.plummer_sphere(32768, seed=778)
    params = c["params"]
    ref = oracle.run(c, params)["particles"]
    t = GradhSphTree(params, precision="mixed")
    t.set_particles(c)
    t.set_tuning(near_depth=64, cell_depth=64, gather_depth=64)
    t.step()
    st = t.stats()
    got = t.results()
    with pytest.raises(GandalfError):
        t.set_tuning(near_depth=32)
    t.close()
    assert st["heavy_forces"] > 0 and st["heavy_density"] > 0
    check_mixed(got, ref)
