"""The oracle (CPU restatement) against fixtures produced by the reference itself."""
import numpy as np
import pytest

from oracle import oracle
from gandalf_gb300.sph import list_hash
from parity import assert_close, check_fp64, check_stars, csr_lists, load_golden, same_lists, star_results


@pytest.mark.parametrize("name,gravity", [("cube2048", False), ("plummer2048", True), ("plummer_stars2048", True)])
def test_oracle_matches_reference_fixture(name, gravity):
    ics, params, ref, d = load_golden(name)
    r = oracle.run(ics, params, lists=True, nthreads=2)
    check_fp64(r["particles"], ref, gravity)
    # KD-tree: same cells (counts and geometry bit-exact; sums to rounding)
    cells = r["cells"]
    gcells = d["cells"]
    assert np.array_equal(cells["N"], gcells[:, 0])
    for k, col in (("bbmin0", 4), ("bbmax2", 9), ("rcell1", 17), ("rmax", 23), ("cdistsqd", 25)):
        assert np.array_equal(cells[k], gcells[:, col]), k
    # leaf membership
    order = r["order"]
    first = cells["first"].astype(int)
    ref_leaves = csr_lists(d["leaf_off"], d["leaf_ids"])
    for lc, mem in zip(d["leaf_cell"], ref_leaves):
        assert np.array_equal(np.sort(order[first[lc]:first[lc] + int(cells["N"][lc])]), mem)
    # SPH neighbour lists are bit-exact
    assert same_lists(r["hydro_neib"], csr_lists(d["hydro_off"], d["hydro_ids"])) == []
    if gravity:
        cnt = np.array([len(l) for l in r["grav_direct"]])
        hsh = np.array([list_hash(l) for l in r["grav_direct"]], dtype=np.uint64)
        assert np.array_equal(cnt, d["direct_count"])
        assert np.array_equal(hsh, d["direct_hash"])
        mine = {int(l): (len(g), list_hash(g)) for l, g in zip(r["gcell_leaf"], r["gcell_lists"])}
        for l, c, h in zip(d["gcell_leaf"], d["gcell_count"], d["gcell_hash"]):
            assert mine[int(l)] == (c, h)


def test_oracle_plants_a_mistake_and_sees_it():
    """A perturbed input must move the oracle away from the fixture (the check has teeth)."""
    ics, params, ref, _ = load_golden("cube2048")
    bad = dict(ics)
    bad["u"] = ics["u"] * (1.0 + 1e-9)
    r = oracle.run(bad, params, nthreads=2)
    with pytest.raises(AssertionError):
        check_fp64(r["particles"], ref, False)


def test_oracle_star_coupling_matches_reference():
    """Gas <- star terms (including the conservative zeta term of the h solve), gpot_hydro
    without the stars, and star <- gas forces (a, adot, gpot) against the reference."""
    ics, params, ref, d = load_golden("plummer_stars2048")
    r = oracle.run(ics, params, nthreads=2)
    assert_close("gpot_hydro", r["particles"]["gpot_hydro"], ref["gpot_hydro"], 1e-11)
    check_stars(r["stars"], star_results(d))
    # the stars matter: without them the gas potential is off by far more than the tolerance
    no_stars = dict(ics)
    no_stars.pop("stars")
    r0 = oracle.run(no_stars, params, nthreads=2)
    with pytest.raises(AssertionError):
        assert_close("gpot", r0["particles"]["gpot"], ref["gpot"], 1e-6)
