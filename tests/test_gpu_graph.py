"""The CUDA-graph step gives exactly the results of the stream-launched step."""
import numpy as np
import pytest

from gandalf_gb300 import ics as ics_mod
from gandalf_gb300.sph import GradhSphTree
from oracle import oracle
from parity import check_fp64

pytestmark = pytest.mark.gpu


def results(t):
    r = t.results()
    r.update({"star_" + k: v for k, v in (t.star_forces().items() if t.nstar else [])})
    return r


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_graph_step_equals_stream_step(precision):
    c = ics_mod.with_stars(ics_mod.plummer_sphere(20000, seed=21), 5, h=0.03, seed=22)
    params = c.pop("params")
    a = GradhSphTree(params, precision=precision)
    a.set_particles(c)
    a.step()
    ra = results(a)
    b = GradhSphTree(params, precision=precision)
    b.set_particles(c)
    for _ in range(3):      # capture, then replays
        b.step(graph=True)
        rb = results(b)
        for k in ra:
            np.testing.assert_array_equal(rb[k], ra[k], err_msg=k)
    assert b.stats()["launches"] == a.stats()["launches"]
    a.close()
    b.close()


def test_graph_follows_new_particles_and_sizes():
    t = GradhSphTree(ics_mod.plummer_sphere(64)["params"])
    for n, seed in ((4099, 1), (4099, 2), (9000, 3)):
        c = ics_mod.plummer_sphere(n, seed=seed)
        params = c.pop("params")
        t.set_particles(c)
        t.step(graph=True)
        check_fp64(t.results(), oracle.run(c, params)["particles"], True)
    t.close()
