"""GPU (fp64 form) against the reference fixtures and the oracle, through the C ABI.

Values: the FP64_TOL tolerances in tests/parity.py.  Lists: bit-exact — the SPH
neighbour list of every particle, the direct-sum partner set (count and hash) of every
particle, the multipole cell set (count and hash) of every leaf, and the KD-tree itself.
"""
import numpy as np
import pytest

from gandalf_gb300 import ics as ics_mod
from gandalf_gb300.sph import GandalfError, GradhSphTree, list_hash
from oracle import oracle
from parity import check_fp64, csr_lists, gradh_record_dtype, load_golden, same_lists

pytestmark = pytest.mark.gpu


def run_gpu(ics, params, record=True, max_sph=4096, precision="fp64"):
    t = GradhSphTree(params, precision=precision)
    t.set_particles(ics)
    if record:
        t.set_recording(True, max_sph)
    t.step()
    out = t.results()
    return t, out


def check_tree(t, d_cells, leaf_cell, leaf_lists):
    tr = t.tree()
    cells = tr["cells"]
    assert np.array_equal(tr["cell_n"], d_cells[:, 0].astype(np.int32))
    # geometry bit-exact: bb, rcell, rmax, cdistsqd (reference columns 4-9, 16-18, 23, 25)
    assert np.array_equal(cells[:, 6:12], d_cells[:, 4:10])
    assert np.array_equal(cells[:, 18:21], d_cells[:, 16:19])
    assert np.array_equal(cells[:, 3], d_cells[:, 23])
    assert np.array_equal(cells[:, 5], d_cells[:, 25])
    # mass and centre of mass to rounding
    np.testing.assert_allclose(cells[:, 2], d_cells[:, 22], rtol=1e-13, atol=0)
    order = tr["order"]
    for lc, mem in zip(leaf_cell, leaf_lists):
        f = tr["cell_first"][lc]
        assert np.array_equal(np.sort(order[f:f + tr["cell_n"][lc]]), mem)


@pytest.mark.parametrize("name,gravity", [("cube2048", False), ("plummer2048", True)])
def test_gpu_matches_reference_fixture(name, gravity):
    ics, params, ref, d = load_golden(name)
    t, out = run_gpu(ics, params)
    check_fp64(out, ref, gravity)
    check_tree(t, d["cells"], d["leaf_cell"], csr_lists(d["leaf_off"], d["leaf_ids"]))
    assert same_lists(t.sph_neighbours(), csr_lists(d["hydro_off"], d["hydro_ids"])) == []
    if gravity:
        cnt, hsh = t.direct_summary()
        assert np.array_equal(cnt, d["direct_count"])
        assert np.array_equal(hsh, d["direct_hash"])
        leaf, ccnt, chsh = t.cell_summary()
        mine = {int(l): (int(c), int(h)) for l, c, h in zip(leaf, ccnt, chsh)}
        for l, c, h in zip(d["gcell_leaf"], d["gcell_count"], d["gcell_hash"]):
            assert mine[int(l)] == (int(c), int(h))
    t.close()


def compare_with_oracle(c, params, gravity):
    r = oracle.run(c, params, summary=True)
    t, out = run_gpu(c, params)
    check_fp64(out, r["particles"], gravity)
    assert same_lists(t.sph_neighbours(), r["hydro_neib"]) == []
    if gravity:
        cnt, hsh = t.direct_summary()
        assert np.array_equal(cnt, r["direct_count"])
        assert np.array_equal(hsh, r["direct_hash"])
        leaf, ccnt, chsh = t.cell_summary()
        assert np.array_equal(leaf, r["leaf_cell"])
        assert np.array_equal(ccnt, r["cell_count"])
        assert np.array_equal(chsh, r["cell_hash"])
    st = t.stats()
    assert st["hydro_pairs"] == r["counts"]["hydro_pairs"]
    if gravity:
        assert st["direct_pairs"] == r["counts"]["direct_pairs"]
        assert st["cell_pairs"] == r["counts"]["cell_pairs"]
    t.close()


def test_gpu_periodic_cube_full_size_vs_oracle():
    """The periodic-cube workload at its full size, N = 32768."""
    c = ics_mod.periodic_cube(32768, seed=1234)
    compare_with_oracle(c, c["params"], gravity=False)


@pytest.mark.parametrize("n", [1000, 4099, 65536])
def test_gpu_plummer_vs_oracle(n):
    """Ragged (non power-of-two) and larger Plummer spheres."""
    c = ics_mod.plummer_sphere(n, seed=77 + n)
    compare_with_oracle(c, c["params"], gravity=True)


def test_gpu_tree_near_tie_coordinates_vs_oracle():
    """x and y of groups of particles agree in all but the lowest mantissa bits (the
    presort orders the top 48 bits of the coordinate keys by radix passes and then puts
    each run of equal top bits into full-key order): tree, lists and values against the
    oracle.  Offsets within a group are distinct, so no two coordinates are equal."""
    c = ics_mod.plummer_sphere(4099, seed=321)
    rng = np.random.default_rng(5)
    for k in ("x", "y"):
        g = np.linspace(-1.0, 1.0, 64)[rng.integers(0, 64, len(c[k]))]
        off = np.zeros(len(g), dtype=np.int64)
        for v in np.unique(g):
            sel = np.flatnonzero(g == v)
            off[sel] = rng.permutation(len(sel))
        c[k] = (g.view(np.int64) + off).view(np.float64)
        assert len(np.unique(c[k])) == len(g)
    compare_with_oracle(c, c["params"], gravity=True)


@pytest.mark.parametrize("n", [5, 9, 100])
def test_gpu_tiny_open_sets(n):
    """Tiny sets: a single-leaf tree and leaves with one particle."""
    c = ics_mod.plummer_sphere(n, seed=5 + n)
    compare_with_oracle(c, dict(c["params"], nleafmax=8), gravity=True)
    compare_with_oracle(c, dict(c["params"], nleafmax=1), gravity=True)


def test_gpu_isolated_particle_terminates():
    """One isolated particle has no h-rho fixed point (its density is the self term
    only, so h_fac (m/rho)^(1/3) grows with h); the reference would redo the cell
    forever.  The GPU step must return, with an error or a bounded result."""
    c = ics_mod.plummer_sphere(1, seed=1)
    t = GradhSphTree(c["params"])
    t.set_particles(c)
    try:
        t.step()
    except GandalfError as e:
        assert "CAPACITY" in str(e) or "NOT_CONVERGED" in str(e)


def test_gpu_step_equals_separate_calls():
    c = ics_mod.plummer_sphere(4096, seed=3)
    _, a = run_gpu(c, c["params"], record=False)
    t = GradhSphTree(c["params"])
    t.set_particles(c)
    t.BuildTree()
    t.UpdateAllSphProperties()
    t.UpdateAllSphForces()
    b = t.results()
    for k in a:
        assert np.array_equal(a[k], b[k]), k


def test_gpu_call_order_is_enforced():
    c = ics_mod.periodic_cube(512, seed=3)
    t = GradhSphTree(c["params"])
    t.set_particles(c)
    with pytest.raises(GandalfError, match="STATE"):
        t.UpdateAllSphHydroForces()
    t.BuildTree()
    with pytest.raises(GandalfError, match="STATE"):
        t.UpdateAllSphHydroForces()
    t.UpdateAllSphProperties()
    t.UpdateAllSphHydroForces()
    with pytest.raises(GandalfError, match="STATE"):
        t.UpdateAllSphForces()   # self_gravity is off


def test_gpu_rejects_bad_particles():
    c = ics_mod.periodic_cube(256, seed=3)
    t = GradhSphTree(c["params"])
    bad = dict(c)
    bad["m"] = c["m"].copy()
    bad["m"][7] = 0.0
    with pytest.raises(GandalfError, match="INVALID"):
        t.set_particles(bad)
    bad = dict(c)
    bad["x"] = c["x"].copy()
    bad["x"][3] = 1.5   # outside the periodic box
    with pytest.raises(GandalfError, match="INVALID"):
        t.set_particles(bad)


def aos_offsets(dt):
    off = {k: dt.fields[k][1] for k in ("r", "v", "m", "h", "u", "rho", "invomega", "zeta", "hfactor",
                                         "hrangesqd", "pressure", "sound", "div_v", "dudt", "a",
                                         "atree", "gpot", "gpot_hydro")}
    return off


def test_gpu_aos_records_roundtrip():
    """The array-of-structures path gives the same results and leaves other fields alone."""
    c = ics_mod.plummer_sphere(3000, seed=9)
    _, soa = run_gpu(c, c["params"], record=False)
    dt = gradh_record_dtype()
    rec = np.zeros(len(c["x"]), dtype=dt)
    rec["r"] = np.stack([c["x"], c["y"], c["z"]], 1)
    rec["v"] = np.stack([c["vx"], c["vy"], c["vz"]], 1)
    rec["m"], rec["u"], rec["h"] = c["m"], c["u"], c["h"]
    rec["iorig"] = np.arange(len(rec))
    rec["alpha"] = 1.0
    t = GradhSphTree(c["params"])
    off = aos_offsets(dt)
    t.set_particles_aos(rec, off)
    t.step()
    t.get_particles_aos(rec, off)
    assert np.array_equal(rec["h"], soa["h"])
    assert np.array_equal(rec["rho"], soa["rho"])
    assert np.array_equal(rec["a"][:, 0], soa["ax"])
    assert np.array_equal(rec["atree"][:, 2], soa["agz"])
    assert np.array_equal(rec["dudt"], soa["dudt"])
    assert np.array_equal(rec["iorig"], np.arange(len(rec)))
    assert np.all(rec["alpha"] == 1.0)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_gravity_lists_as_full_sets(precision):
    """Direct-sum partners per particle and multipole cells per leaf compared as full sets
    with the oracle's lists (beside the count-and-hash summaries used at large N).  The
    mixed form is compared with the oracle run on its own smoothing lengths."""
    c = ics_mod.plummer_sphere(3000, seed=3001)
    params = c["params"]
    t = GradhSphTree(params, precision=precision)
    t.set_particles(c)
    t.set_recording(True, 1024)
    t.set_list_recording(4096, 4096)
    t.step()
    got = t.results()
    dl = t.direct_lists()
    leaves, _, _ = t.cell_summary()
    cl = t.cell_lists()
    t.close()
    given = None if precision == "fp64" else {k: got[k] for k in ("h", "rho", "invomega", "zeta", "pressure", "sound")}
    r = oracle.run(c, params, lists=True, given=given)
    assert same_lists(dl, r["grav_direct"]) == []
    ref_cells = {int(l): np.sort(g) for l, g in zip(r["gcell_leaf"], r["gcell_lists"])}
    assert len(ref_cells) == len(leaves)
    for leaf, cells in zip(leaves, cl):
        np.testing.assert_array_equal(np.sort(cells), ref_cells[int(leaf)])
    assert sum(len(x) for x in dl) > 0 and sum(len(x) for x in cl) > 0


@pytest.mark.parametrize("nleafmax", [1, 32])
def test_mixed_lists_at_extreme_leaf_sizes(nleafmax):
    """The mixed form's near and direct-sum lists hold each leaf as one word (first slot and
    count): at one particle a leaf and at 32 (one lane a particle) the lists are the
    oracle's as full sets, the oracle run on the mixed form's own smoothing lengths."""
    c = ics_mod.plummer_sphere(3000, seed=3100 + nleafmax)
    params = dict(c["params"], nleafmax=nleafmax)
    t = GradhSphTree(params, precision="mixed")
    t.set_particles(c)
    t.set_recording(True, 1024)
    t.set_list_recording(8192, 8192)
    t.step()
    got = t.results()
    dl = t.direct_lists()
    leaves, _, _ = t.cell_summary()
    cl = t.cell_lists()
    nb = t.sph_neighbours()
    t.close()
    given = {k: got[k] for k in ("h", "rho", "invomega", "zeta", "pressure", "sound")}
    r = oracle.run(c, params, lists=True, given=given)
    assert same_lists(nb, r["hydro_neib"]) == []
    assert same_lists(dl, r["grav_direct"]) == []
    ref_cells = {int(l): np.sort(g) for l, g in zip(r["gcell_leaf"], r["gcell_lists"])}
    mine = {int(l): np.sort(g) for l, g in zip(leaves, cl)}
    # the complete tree's empty leaves (no particle, so no walk) appear on this side only
    assert set(ref_cells) <= set(mine)
    for leaf, cells in mine.items():
        if leaf in ref_cells:
            np.testing.assert_array_equal(cells, ref_cells[leaf])
        else:
            assert len(cells) == 0
