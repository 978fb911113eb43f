"""Batched stepping of many simulations against stepping each one on its own.

The batch runs the same per-leaf device code as the single-simulation kernels, so with
the same lanes per particle (leaves of 5-8 particles everywhere here) every result is
bit-identical to the simulation's own step; one box is also checked against the oracle.
"""
import numpy as np
import pytest

from gandalf_gb300 import ics as ics_mod
from gandalf_gb300.sph import GradhSphBatch, GradhSphTree
from oracle import oracle
from parity import check_mixed

pytestmark = pytest.mark.gpu


def make(c):
    params = c.pop("params")
    t = GradhSphTree(params, precision="mixed")
    t.set_particles(c)
    return t, params


def compare(sets):
    solo, trees = [], []
    for c in sets:
        t, _ = make(dict(c))
        t.step()
        solo.append((t.results(), t.stats()))
        t.close()
        trees.append(make(dict(c))[0])
    b = GradhSphBatch(trees)
    for rep in range(2):          # capture, then a replay
        b.step()
        for (r0, s0), t in zip(solo, trees):
            r1, s1 = t.results(), t.stats()
            for k in r0:
                np.testing.assert_array_equal(r1[k], r0[k], err_msg=k)
            for k in ("density_pairs", "hydro_pairs", "direct_pairs", "cell_pairs"):
                assert s1[k] == s0[k], k
    st = b.stats()
    assert st["ms"] > 0 and st["launches"] > 0
    b.close()
    for t in trees:
        t.close()


def test_kh_batch_equals_single_steps():
    compare([ics_mod.kh_box(n, seed=s) for n, s in ((4096, 1), (5000, 2), (9000, 3), (20000, 4), (7000, 5))])


def test_gravity_batch_equals_single_steps():
    compare([ics_mod.plummer_sphere(n, seed=s) for n, s in ((4099, 6), (6000, 7), (16384, 8))])


def test_kh_box_against_oracle():
    c = ics_mod.kh_box(8192, seed=9)
    params = dict(c["params"])
    t, _ = make(dict(c))
    b = GradhSphBatch([t])
    b.step()
    ref = oracle.run({k: v for k, v in c.items() if k != "params"}, params)["particles"]
    check_mixed(t.results(), ref)
    b.close()
    t.close()


def test_largest_ensemble_box_inside_a_batch_against_oracle():
    """The largest box of the 64-box ensemble (about 129k particles) stepped inside a batch
    with the smallest and a middle-sized box, against the oracle."""
    boxes = ics_mod.kh_ensemble(64, 4096, 131072, seed=2024)
    sizes = [len(b["x"]) for b in boxes]
    order = np.argsort(sizes)
    pick = [boxes[order[0]], boxes[order[len(order) // 2]], boxes[order[-1]]]
    trees = [make(dict(c))[0] for c in pick]
    b = GradhSphBatch(trees)
    b.step()
    big = pick[-1]
    assert len(big["x"]) > 120000
    ref = oracle.run({k: v for k, v in big.items() if k != "params"}, dict(big["params"]))["particles"]
    print(len(big["x"]), check_mixed(trees[-1].results(), ref))
    b.close()
    for t in trees:
        t.close()
